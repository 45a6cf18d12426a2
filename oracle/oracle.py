"""ctypes binding of the CPU oracle (oracle/kpm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker.  The product library
never imports this module.  Parity unpinned against the reference's own
outputs (see kpm_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libkpm_oracle.so"

MODE_SPARSE, MODE_PERIODIC_BARE, MODE_BARE = 0, 1, 2
GAUGE_NONE, GAUGE_LINEAR, GAUGE_SITE = 0, 1, 2
K_DIRICHLET, K_FEJER, K_LORENTZ, K_JACKSON, K_LANCZOS, K_WANG_ZUNGER = range(6)


class Lattice(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n_atoms", C.c_int32),
        ("span", C.c_int32 * 3), ("extend", C.c_int32 * 3),
        ("bases", C.c_void_p), ("atom_pos", C.c_void_p),
        ("n_hops", C.c_int32),
        ("hop_from", C.c_void_p), ("hop_to", C.c_void_p), ("hop_latv", C.c_void_p), ("hop_t", C.c_void_p),
        ("mode", C.c_int32), ("is_complex", C.c_int32), ("gauge_kind", C.c_int32),
        ("gauge_linear", C.c_void_p), ("gauge_site", C.c_void_p), ("scalar_site", C.c_void_p),
        ("removed", C.c_void_p),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        L = C.CDLL(str(LIB_PATH))
        vp, i32, i64, d, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_double, C.c_uint64
        sig = {
            "tbo_u01": (d, [u64, u64, u64]),
            "tbo_random_phase_kets": (None, [i32, i32, u64, vp]),
            "tbo_uniform_disorder": (None, [i32, d, u64, vp]),
            "tbo_nn_shell": (i32, [i32, vp, i32, vp, i32, i32, vp, vp, i32]),
            "tbo_total_sites": (i64, [vp]),
            "tbo_triplet_bound": (i64, [vp]),
            "tbo_build_csc": (i64, [vp, vp, vp, vp, i64]),
            "tbo_position_diag": (i64, [vp, i32, vp]),
            "tbo_rescale_csc": (i64, [i32, vp, vp, vp, i32, d, d, vp, vp, vp, i64]),
            "tbo_commutator_values": (None, [i32, vp, vp, vp, i32, vp, vp]),
            "tbo_csc_mult": (None, [i32, vp, vp, vp, i32, i32, vp, vp]),
            "tbo_cheb_moments": (i32, [i32, vp, vp, vp, i32, i32, vp, vp, i32, vp, i32, i32]),
            "tbo_trace_braket": (d, [i32, i32, vp, vp]),
            "tbo_trace_braket_complex": (None, [i32, i32, vp, vp, vp]),
            "tbo_cheb_blocks": (i32, [i32, vp, vp, vp, i32, i32, vp, i32, vp]),
            "tbo_kernel_seq": (None, [i32, i32, d, d, vp]),
            "tbo_expn_coef_alpha_seq": (None, [d, d, i32, vp]),
            "tbo_green_imag_eval": (d, [i32, vp, vp, d, d]),
            "tbo_green_imag_fft": (None, [i32, vp, vp, i32, vp, vp]),
            "tbo_mu_nm": (None, [i32, i64, vp, vp, vp]),
            "tbo_bastin_zeta": (None, [i32, vp, i32, vp, d, vp]),
            "tbo_greenwood_sigma": (None, [i32, vp, i32, vp, d, vp]),
            "tbo_bastin_integrate": (i32, [i32, vp, vp, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class LatticeSpec:
    """Owns the numpy buffers behind a tbo_lattice."""

    def __init__(self, dim, span, bases, atom_pos, hop_from, hop_to, hop_latv, hop_t, mode=MODE_SPARSE,
                 is_complex=True, extend=None, gauge_linear=None, gauge_site=None, scalar_site=None, removed=None):
        self.bases = np.ascontiguousarray(np.asarray(bases, dtype=np.float64).T.reshape(-1))  # 3 x dim col-major
        self.atom_pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        self.hop_from = np.ascontiguousarray(hop_from, dtype=np.int32)
        self.hop_to = np.ascontiguousarray(hop_to, dtype=np.int32)
        self.hop_latv = np.ascontiguousarray(hop_latv, dtype=np.int32).reshape(-1)
        t = np.asarray(hop_t, dtype=np.complex128)
        self.hop_t = np.ascontiguousarray(np.stack([t.real, t.imag], axis=1)).reshape(-1)
        self.gauge_linear = None if gauge_linear is None else np.ascontiguousarray(gauge_linear, dtype=np.float64)
        self.gauge_site = None if gauge_site is None else np.ascontiguousarray(gauge_site, dtype=np.float64)
        self.scalar_site = None if scalar_site is None else np.ascontiguousarray(scalar_site, dtype=np.float64)
        self.removed = None if removed is None else np.ascontiguousarray(removed, dtype=np.int32)
        s = Lattice()
        s.dim = dim
        s.n_atoms = len(self.atom_pos) // 3
        for i in range(3):
            s.span[i] = span[i] if i < dim else 1
            s.extend[i] = (extend[i] if extend is not None and i < dim else 0)
        s.bases, s.atom_pos = _p(self.bases), _p(self.atom_pos)
        s.n_hops = len(self.hop_from)
        s.hop_from, s.hop_to, s.hop_latv, s.hop_t = _p(self.hop_from), _p(self.hop_to), _p(self.hop_latv), _p(self.hop_t)
        s.mode, s.is_complex = mode, int(is_complex)
        s.gauge_kind = GAUGE_LINEAR if gauge_linear is not None else (GAUGE_SITE if gauge_site is not None else GAUGE_NONE)
        s.gauge_linear, s.gauge_site = _p(self.gauge_linear), _p(self.gauge_site)
        s.scalar_site, s.removed = _p(self.scalar_site), _p(self.removed)
        self.s = s

    def ref(self):
        return C.byref(self.s)


def build_csc(spec: LatticeSpec):
    L = lib()
    N = L.tbo_total_sites(spec.ref())
    cap = L.tbo_triplet_bound(spec.ref()) + 1
    cp = np.zeros(N + 1, dtype=np.int32)
    ri = np.zeros(cap, dtype=np.int32)
    v = np.zeros(cap, dtype=np.complex128 if spec.s.is_complex else np.float64)
    nnz = L.tbo_build_csc(spec.ref(), _p(cp), _p(ri), _p(v), cap)
    assert nnz >= 0
    return cp, ri[:nnz].copy(), v[:nnz].copy()


def position_diag(spec: LatticeSpec, axis: int):
    L = lib()
    N = L.tbo_total_sites(spec.ref())
    x = np.zeros(N)
    k = L.tbo_position_diag(spec.ref(), axis, _p(x))
    return x[:k]


def rescale_csc(n, cp, ri, v, a, b):
    cplx = np.iscomplexobj(v)
    cap = len(ri) + n + 1
    ocp = np.zeros(n + 1, dtype=np.int32)
    ori = np.zeros(cap, dtype=np.int32)
    ov = np.zeros(cap, dtype=np.complex128 if cplx else np.float64)
    v = np.ascontiguousarray(v)
    nnz = lib().tbo_rescale_csc(n, _p(cp), _p(ri), _p(v), int(cplx), a, b, _p(ocp), _p(ori), _p(ov), cap)
    assert nnz >= 0
    return ocp, ori[:nnz].copy(), ov[:nnz].copy()


def commutator_values(n, cp, ri, v, x):
    cplx = np.iscomplexobj(v)
    out = np.zeros_like(v)
    v = np.ascontiguousarray(v)
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().tbo_commutator_values(n, _p(cp), _p(ri), _p(v), int(cplx), _p(x), _p(out))
    return out


def random_phase_kets(n, R, seed):
    out = np.zeros((n, R), dtype=np.complex128, order="F")
    lib().tbo_random_phase_kets(n, R, seed, _p(out))
    return out


def uniform_disorder(n, W, seed):
    out = np.zeros(n)
    lib().tbo_uniform_disorder(n, W, seed, _p(out))
    return out


def cheb_moments(n, cp, ri, v, n_mom, bras, kets, threads=0, steps_limit=0):
    cplx = np.iscomplexobj(v)
    v = np.ascontiguousarray(v)
    kets = np.asfortranarray(kets, dtype=np.complex128)
    bras = kets if bras is None else np.asfortranarray(bras, dtype=np.complex128)
    mu = np.zeros(n_mom)
    rc = lib().tbo_cheb_moments(n, _p(cp), _p(ri), _p(v), int(cplx), n_mom, _p(bras), _p(kets), kets.shape[1],
                                _p(mu), threads, steps_limit)
    if rc != 0:
        raise ValueError("oracle: n must be >= 2")
    return mu


def cheb_blocks(n, cp, ri, v, n_mom, x0):
    cplx = np.iscomplexobj(v)
    v = np.ascontiguousarray(v)
    x0 = np.asfortranarray(x0, dtype=np.complex128)
    out = np.zeros((n_mom, x0.shape[1], n), dtype=np.complex128)   # block k: column-major N x R
    lib().tbo_cheb_blocks(n, _p(cp), _p(ri), _p(v), int(cplx), n_mom, _p(x0), x0.shape[1], _p(out))
    return out


def cheb_expand(n, cp, ri, v, coef, x0):
    """sum_k coef[k] T_k(H) x0: the Cheb_first_kind_seq_view walk with a host
    sum (TB/numerical.h:346-361, used as in TB/snippets.h:194-217)."""
    blocks = cheb_blocks(n, cp, ri, v, len(coef), x0)        # (K, R, n)
    out = np.tensordot(np.asarray(coef, dtype=np.complex128), blocks, axes=(0, 0))
    return np.asfortranarray(out.T)


def delta_coefficients(e, N):
    """a_d(k) T_k(e) for k = 0 .. N, the view loop of TB/snippets.h:194-202
    (Cheb_first_kind_seq_view(e, 1.) yields T_0 .. T_N before i reaches N)."""
    t0, t1 = 1.0, e
    c = []
    for k in range(N + 1):
        c.append((1.0 if k == 0 else 2.0) * t0)
        t0, t1 = t1, 2.0 * e * t1 - t0
    return np.asarray(c, dtype=np.complex128)


def kernel_seq(kind, N, p0=0.0, p1=0.0):
    g = np.zeros(N)
    lib().tbo_kernel_seq(kind, N, p0, p1, _p(g))
    return g


def expn_coef_alpha_seq(z, n):
    out = np.zeros(2 * n)
    z = complex(z)
    lib().tbo_expn_coef_alpha_seq(z.real, z.imag, n, _p(out))
    return out.view(np.complex128)


def green_imag_eval(g, mu, z):
    g = np.ascontiguousarray(g, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    return np.array([lib().tbo_green_imag_eval(len(mu), _p(g), _p(mu), complex(x).real, complex(x).imag)
                     for x in np.atleast_1d(z)])


def green_imag_fft(g, mu, upsample=1):
    g = np.ascontiguousarray(g, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    N = len(mu) * upsample
    E = np.zeros(N)
    v = np.zeros(N)
    lib().tbo_green_imag_fft(len(mu), _p(g), _p(mu), upsample, _p(E), _p(v))
    return E, v


def nn_shell(dim, bases, atom_pos, from_, nn, cap=512):
    b = np.ascontiguousarray(np.asarray(bases, dtype=np.float64).T.reshape(-1))
    p = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
    to = np.zeros(cap, dtype=np.int32)
    lv = np.zeros(3 * cap, dtype=np.int32)
    k = lib().tbo_nn_shell(dim, _p(b), len(p) // 3, _p(p), from_, nn, _p(to), _p(lv), cap)
    assert k >= 0
    return to[:k].copy(), lv[: 3 * k].reshape(k, 3).copy()


def mu_nm(L_blocks, R_blocks):
    """L_blocks, R_blocks: (M, K) complex arrays."""
    Lb = np.ascontiguousarray(L_blocks, dtype=np.complex128)
    Rb = np.ascontiguousarray(R_blocks, dtype=np.complex128)
    M, K = Lb.shape
    out = np.zeros((M, M), dtype=np.complex128)
    lib().tbo_mu_nm(M, K, _p(Lb), _p(Rb), _p(out))
    return out


def bastin_zeta(mu, eps, vol=1.0):
    mu = np.ascontiguousarray(mu, dtype=np.complex128)
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    out = np.zeros(len(eps), dtype=np.complex128)
    lib().tbo_bastin_zeta(mu.shape[0], _p(mu), len(eps), _p(eps), vol, _p(out))
    return out


def greenwood_sigma(mu, eps, R):
    mu = np.ascontiguousarray(mu, dtype=np.complex128)
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    out = np.zeros(len(eps))
    lib().tbo_greenwood_sigma(mu.shape[0], _p(mu), len(eps), _p(eps), float(R), _p(out))
    return out


def bastin_integrate(eps, zeta):
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    zeta = np.ascontiguousarray(zeta, dtype=np.complex128)
    N = len(eps)
    E, re, im = np.zeros(N), np.zeros(N), np.zeros(N)
    n = lib().tbo_bastin_integrate(N, _p(eps), _p(zeta), _p(E), _p(re), _p(im))
    return E[:n], re[:n], im[:n]


def kubo_mu(n, cp, ri, v, M, kets, AL=None, BL=None, AR=None, BR=None, g=None):
    """mu_mn = sum conj(g_m AL T_m BL r) (g_n AR T_n BR r) in FP64; operators are
    (cp, ri, v) CSC triples or None."""
    def app(op, X):
        if op is None:
            return X
        ocp, ori, ov = op
        Y = np.zeros_like(X)
        lib().tbo_csc_mult(n, _p(ocp), _p(ori), _p(np.ascontiguousarray(ov)), int(np.iscomplexobj(ov)), X.shape[1],
                           _p(np.asfortranarray(X)), _p(Y))
        return Y

    kets = np.asfortranarray(kets, dtype=np.complex128)
    R = kets.shape[1]

    def side(A, B):
        x0 = np.asfortranarray(app(B, kets))
        blocks = cheb_blocks(n, cp, ri, v, M, x0)               # (M, R, n)
        out = np.zeros((M, R * n), dtype=np.complex128)
        for m in range(M):
            blk = np.asfortranarray(blocks[m].T)                  # n x R
            out[m] = np.asfortranarray(app(A, blk)).T.reshape(-1)
        return out

    Lb = side(AL, BL)
    Rb = side(AR, BR)
    mu = mu_nm(Lb, Rb)
    if g is not None:
        mu = mu * np.outer(g, g)
    return mu
