"""Kubo conductivities from double-Chebyshev moments, backed by libtbk.

    kubo_mu                       mu_mn of stored Chebyshev blocks (TB/snippets.h:326-342)
    conductivity_Kubo_Bastin      sigma_xy, TB/snippets.h:306-456
    conductivity_spectrum         Kubo-Greenwood sigma_xx(E), TB/snippets.h:225-304
    generate_V_moments            explicit velocity moments, TB/snippets.h:491-518
    conductivity_test_sawtooth    single-energy delta projection, TB/snippets.h:173-223
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import capi
from .capi import check, lib
from .kpm import GreenFunction, Kernel, Lorentz, Dirichlet, _block
from .lattice import PartialLattice, SparseMatrix, commutator


def _h(op):
    return None if op is None else op.handle


_RECURSION = {"fp64": 0, "mixed": capi.MU_MIXED_RECURSION, "dd": capi.MU_DD_RECURSION}


def kubo_mu(Ht: SparseMatrix, AL=None, BL=None, AR=None, BR=None, M: int = 64, R: int = 4, seed: int = 0,
            kets=None, kernel: Kernel | None = None, tensor: bool = False, budget_gb: float = 0.0,
            recursion: str = "mixed", fuse_ops: bool = False, both_sides: bool = False,
            fp64_blocks: bool = False) -> np.ndarray:
    """mu_mn = sum conj(g_m AL T_m BL r) (g_n AR T_n BR r); operators None = identity.
    recursion: "mixed" (default: complex64 work blocks, FP32 H~; the stored
    blocks are complex64 either way, and against the FP64 reference form the
    sigma errors are the same as with the wider recursions), "dd" (double-float
    work blocks: FP64-class recursion on the FP32 pipe) or "fp64" (complex128).  fuse_ops:
    form AL / AR products inside the recursion step when they share H~'s
    sparsity (same stored bits, one pass instead of two; opt-in, measured no
    faster); both_sides (with fuse_ops): run the two sides as one recursion of
    twice the width (same bits).  fp64_blocks: the FP64 reference form —
    complex128 stored blocks and an FP64 GEMM (tensor, fuse_ops and both_sides
    are then ignored)."""
    kernel = kernel if kernel is not None else Dirichlet()
    mu = np.zeros((M, M), dtype=np.complex128)
    K = None
    if kets is not None:
        K = _block(kets, Ht.shape[0])
        R = K.shape[1]
    check(lib().tbk_kubo_mu(Ht.handle, _h(AL), _h(BL), _h(AR), _h(BR), M, R, int(seed),
                            None if K is None else capi.ptr(K), kernel.kind, kernel.p0, kernel.p1,
                            (capi.MU_TENSOR if tensor else capi.MU_CUDA_CORE) | _RECURSION[recursion]
                            | (capi.MU_FUSED_OPS if fuse_ops else 0)
                            | (capi.MU_BOTH_SIDES if both_sides else 0)
                            | (capi.MU_FP64_BLOCKS if fp64_blocks else 0),
                            float(budget_gb), capi.ptr(mu), None))
    return mu


def kubo_release() -> None:
    """Return the device memory kubo_mu's pool keeps between calls (stores and
    work blocks of at most 16 GB)."""
    check(lib().tbk_kubo_release())


def mu_from_blocks(L: np.ndarray, R: np.ndarray, tensor: bool = True) -> np.ndarray:
    """mu_mn = sum_k conj(L[m, k]) R[n, k] on the GPU (blocks rounded to complex64)."""
    L = np.ascontiguousarray(L, dtype=np.complex128)
    R = np.ascontiguousarray(R, dtype=np.complex128)
    M, K = L.shape
    mu = np.zeros((M, M), dtype=np.complex128)
    check(lib().tbk_mu_from_blocks(M, K, capi.ptr(L), capi.ptr(R), capi.MU_TENSOR if tensor else capi.MU_CUDA_CORE,
                                   capi.ptr(mu), None))
    return mu


def kubo_last_timing() -> dict:
    a, b, f, by = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    n = C.c_int32()
    check(lib().tbk_kubo_last_timing(C.byref(a), C.byref(b), C.byref(f), C.byref(by), C.byref(n)))
    return {"ms_blocks": a.value, "ms_gemm": b.value, "gemm_flops": f.value, "block_bytes": by.value,
            "chunks": n.value}


def chebyshev_nodes(N: int) -> np.ndarray:
    """eps_k = cos((k + 1/2) pi / N), the nodes of the DCT-III (descending)."""
    return np.cos((np.arange(N) + 0.5) / N * math.pi)


def bastin_zeta(mu: np.ndarray, eps, volume: float = 1.0) -> np.ndarray:
    mu = np.ascontiguousarray(mu, dtype=np.complex128)
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    z = np.zeros(len(eps), dtype=np.complex128)
    check(lib().tbk_kubo_bastin_zeta(mu.shape[0], capi.ptr(mu), len(eps), capi.ptr(eps), float(volume), capi.ptr(z), None))
    return z


def greenwood_sigma(mu: np.ndarray, eps, R: float) -> np.ndarray:
    mu = np.ascontiguousarray(mu, dtype=np.complex128)
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    s = np.zeros(len(eps))
    check(lib().tbk_kubo_greenwood_sigma(mu.shape[0], capi.ptr(mu), len(eps), capi.ptr(eps), float(R), capi.ptr(s), None))
    return s


def bastin_integrate(eps, zeta):
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    zeta = np.ascontiguousarray(zeta, dtype=np.complex128)
    N = len(eps)
    E, re, im = np.zeros(N), np.zeros(N), np.zeros(N)
    n = C.c_int32()
    check(lib().tbk_kubo_bastin_integrate(N, capi.ptr(eps), capi.ptr(zeta), capi.ptr(E), capi.ptr(re), capi.ptr(im),
                                          C.byref(n)))
    return E[: n.value], re[: n.value], im[: n.value]


def conductivity_Kubo_Bastin(H_og: SparseMatrix, op_x: SparseMatrix, op_y: SparseMatrix, N: int, E_min: float,
                             E_max: float, Volume: float = 1.0, R: int = 4, seed: int = 0, kernel: Kernel | None = None,
                             tensor: bool = False, budget_gb: float = 0.0, recursion: str = "mixed", fuse_ops: bool = False,
                             velocity=None, fp64_blocks: bool = False):
    """TB/snippets.h:306-456: G(N, H, E_min-1e-8, E_max+1e-8); v = X H~ - H~ X;
    aL = g T r, aR = g v_x T v_y r; zeta at the N Chebyshev nodes; cumulative
    integral from E = 0.  Returns dict with eps, zeta, E, sigma_re, sigma_im, mu.
    velocity: optional callable G -> (v_x, v_y) replacing the commutators (e.g.
    the bond-displacement form, PartialLattice.op_velocity_bond with scale 1/G.a)."""
    kernel = kernel if kernel is not None else Lorentz(6.0)
    G = GreenFunction(N, H_og, E_min - 1e-8, E_max + 1e-8)
    Ht = G.scaled_HE
    if velocity is not None:
        v_x, v_y = velocity(G)
    else:
        v_x = commutator(Ht, op_x)
        v_y = commutator(Ht, op_y)
    mu = kubo_mu(Ht, None, None, v_x, v_y, N, R, seed, kernel=kernel, tensor=tensor, budget_gb=budget_gb,
                 recursion=recursion, fuse_ops=fuse_ops, fp64_blocks=fp64_blocks)
    eps = chebyshev_nodes(N)
    zeta = bastin_zeta(mu, eps, Volume)
    E, sr, si = bastin_integrate(eps, zeta)
    return {"eps": eps, "zeta": zeta, "E": E, "sigma_re": sr, "sigma_im": si, "mu": mu, "G": G}


def conductivity_spectrum(H_og: SparseMatrix, op_x: SparseMatrix, op_y: SparseMatrix, N: int, R: int = 128,
                          seed: int = 0, kernel: Kernel | None = None, E_min: float = -4.0001, E_max: float = 4.0001,
                          tensor: bool = False, budget_gb: float = 0.0, recursion: str = "mixed", fuse_ops: bool = False,
                          fp64_blocks: bool = False):
    """Kubo-Greenwood spectrum, TB/snippets.h:225-304: aR = g T r, aL = g v_x T v_x r,
    sigma(eps_k) = -<phi_L|phi_R> w(eps_k)^2 / R at the N Chebyshev nodes."""
    kernel = kernel if kernel is not None else Lorentz(6.0)
    G = GreenFunction(N, H_og, E_min, E_max)
    Ht = G.scaled_HE
    v_x = commutator(Ht, op_x)
    mu = kubo_mu(Ht, v_x, v_x, None, None, N, R, seed, kernel=kernel, tensor=tensor, budget_gb=budget_gb,
                 recursion=recursion, fuse_ops=fuse_ops, fp64_blocks=fp64_blocks)
    eps = chebyshev_nodes(N)
    return eps, greenwood_sigma(mu, eps, R), mu


def conductivity_test_sawtooth(X: PartialLattice, N: int, E: float, R: int = 4, seed: int = 0,
                               precision="dd") -> float:
    """TB/snippets.h:173-223: single-energy Kubo-Greenwood value of a sawtooth
    chain.  Real open-BC H, G(N, H, 4t - 2 - 1e-6, 4t + 1e-6) with t = -E/2,
    e = G.scale(E); v_x = X H~ - H~ X; D = sum_{k=0..N} a_d(k) T_k(e) T_k(H~)
    (the view loop runs N + 1 terms); returns Re tr(<v_x D v_x r | D r>) / R.
    Kets: R seeded random-phase vectors (the reference draws unseeded ones)."""
    from .kpm import bases_of_uniform_ampl_with_random_phases, cheb_expand, delta_coefficients, sparse_apply
    H_og = X.get_Hamiltonian_sparse(float)
    t = -E / 2.0
    G = GreenFunction(N, H_og, 4 * t - 2.0 - 1e-6, 4 * t + 1e-6)
    e = G.scale(E, 1.0)
    H = G.scaled_HE
    v_x = commutator(H, X.op_position(0))
    kets = bases_of_uniform_ampl_with_random_phases(X.get_total_number(), R, seed)
    coef = delta_coefficients(e, N)
    kets_R = cheb_expand(H, coef, kets, precision)
    kets_L = sparse_apply(v_x, cheb_expand(H, coef, sparse_apply(v_x, kets, precision), precision), precision)
    return float(np.sum(kets_L.real * kets_R.real + kets_L.imag * kets_R.imag)) / R


def generate_V_moments(X: PartialLattice, N: int, R: int = 100, seed: int = 0, tensor: bool = False) -> np.ndarray:
    """TB/snippets.h:491-518: bare real H, G(N, H, -1.000001, 1.000001), v_x =
    X.op_velocity(0); V_nm = Re <v_x T_n v_x r | T_m r> / R for m >= n (upper
    triangle, zero below)."""
    H = X.get_Hamiltonian_bare_sparse(float)
    G = GreenFunction(N, H, -1.000001, 1.000001)
    v_x = X.op_velocity(0)
    mu = kubo_mu(G.scaled_HE, v_x, v_x, None, None, N, R, seed, kernel=Dirichlet(), tensor=tensor)
    V = np.real(mu) / R
    return np.triu(V)
