"""Moment and result files.

    save_moments / load_moments   binary (tbk_moments_*): 256-byte header with the
                                  bounds, R, seed, kernel and precision, then the
                                  values; checksum checked on load
    output_to_file                the reference's text columns, TB/utils.h:42-69
    write_V_moments_text          generate_V_moments' V_moments.txt, TB/snippets.h:504-517
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import capi
from .capi import check, lib

KINDS = {"dos": capi.MOMENTS_DOS, "mu_nm": capi.MOMENTS_MU_NM, "v_nm": capi.MOMENTS_V_NM}
_KIND_NAMES = {v: k for k, v in KINDS.items()}


def save_moments(path, data, kind: str = "dos", R: int = 0, seed: int = 0, e_min: float = -1.0, e_max: float = 1.0,
                 precision: int = 0, kernel: int = -1, kernel_p0: float = 0.0, kernel_p1: float = 0.0,
                 n_sites: int = 0, label: str = "") -> None:
    a = np.asarray(data)
    cplx = np.iscomplexobj(a)
    a2 = a.reshape(-1, 1) if a.ndim == 1 else a
    if a2.ndim != 2:
        raise ValueError("moments must be a vector or a matrix")
    buf = np.ascontiguousarray(a2, dtype=np.complex128 if cplx else np.float64)
    h = capi.MomentsHeader()
    h.kind = KINDS[kind]
    h.rows, h.cols = buf.shape
    h.is_complex = 1 if cplx else 0
    h.R, h.precision, h.kernel = int(R), int(precision), int(kernel)
    h.seed = int(seed)
    h.e_min, h.e_max = float(e_min), float(e_max)
    h.kernel_p0, h.kernel_p1 = float(kernel_p0), float(kernel_p1)
    h.n_sites = int(n_sites)
    h.label = label.encode()[:159]
    check(lib().tbk_moments_save(os.fsencode(path), C.addressof(h), capi.ptr(buf)))


def load_moments(path):
    """(values, meta): a vector for kind "dos", else a rows x cols matrix."""
    h = capi.MomentsHeader()
    p = os.fsencode(path)
    check(lib().tbk_moments_load_header(p, C.addressof(h)))
    n = h.rows * h.cols * (2 if h.is_complex else 1)
    buf = np.zeros(max(n, 1), dtype=np.float64)
    check(lib().tbk_moments_load(p, C.addressof(h), capi.ptr(buf), n))
    vals = buf[:n].view(np.complex128) if h.is_complex else buf[:n]
    vals = vals.reshape(h.rows, h.cols)
    if h.kind == capi.MOMENTS_DOS:
        vals = vals[:, 0]
    meta = dict(kind=_KIND_NAMES.get(h.kind, h.kind), R=h.R, seed=h.seed, e_min=h.e_min, e_max=h.e_max,
                precision=h.precision, kernel=h.kernel, kernel_p0=h.kernel_p0, kernel_p1=h.kernel_p1,
                n_sites=h.n_sites, label=h.label.decode(), checksum=h.checksum)
    return vals.copy(), meta


def _g(x) -> str:
    """A double as std::ostream writes it by default (six significant digits)."""
    return "%g" % float(x)


def output_to_file(filename, *vectors) -> None:
    """utils::output_to_file (TB/utils.h:42-69): the vectors as columns, every
    element followed by one space, one row per line; a nested element (a row
    of its own) is written element by element.  Unequal sizes: "Not equal size"."""
    sizes = [len(v) for v in vectors]
    if any(s != sizes[0] for s in sizes):
        raise ValueError("Not equal size")
    with open(filename, "w") as out:
        for i in range(sizes[0] if sizes else 0):
            for v in vectors:
                e = v[i]
                if np.ndim(e):
                    out.write("".join(_g(x) + " " for x in np.ravel(e)))
                else:
                    out.write(_g(e) + " ")
            out.write("\n")


def write_V_moments_text(filename, V) -> None:
    """V_moments.txt of generate_V_moments (TB/snippets.h:504-517): row i holds
    i zeros, then V[i, i:], each followed by one space."""
    V = np.asarray(V)
    N = V.shape[0]
    with open(filename, "w") as f:
        for i in range(N):
            f.write("0 " * i + "".join(_g(V[i, j]) + " " for j in range(i, N)) + "\n")
