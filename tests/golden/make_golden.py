"""Generates the golden fixtures in this directory (run: python tests/golden/make_golden.py).

The reference project ships no tests and no data, and cannot be built here, so
its own outputs cannot be recorded.  These fixtures are analytic known answers,
computed here by plane-wave sums that share no code with the oracle or the GPU
library:

  exact_moments.npz
    For periodic lattices with one hopping shell, H~ = H/a is diagonal in
    k-space, so Tr T_n(H~) = sum over k and bands of T_n(eps_b(k)/a).  With the
    N unit vectors as kets (R = N), the KPM moments mu_n equal this trace
    exactly; tests feed the identity block through the oracle and the GPU path.

  counts.json
    Stored-entry counts of H and H~ = (H - bI)/a for the lattices of the
    benchmark configurations (coordination number times sites, plus the
    diagonal that the rescale adds).
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def cheb_trace(eps_over_a: np.ndarray, M: int) -> np.ndarray:
    th = np.arccos(np.clip(eps_over_a, -1.0, 1.0))
    return np.cos(np.outer(np.arange(M), th)).sum(axis=1)


def square(L: int, t: float) -> np.ndarray:
    k = 2 * np.pi * np.arange(L) / L
    return (2 * t * (np.cos(k)[:, None] + np.cos(k)[None, :])).reshape(-1)


def honeycomb(L: int, t: float) -> np.ndarray:
    # 1NN of A: B in cells (0,0), (-1,0), (0,-1) -> |1 + e^{ik1} + e^{ik2}|
    k = 2 * np.pi * np.arange(L) / L
    f = np.abs(1 + np.exp(1j * k)[:, None] + np.exp(1j * k)[None, :]).reshape(-1)
    return np.concatenate([t * f, -t * f])


def fcc(L: int, t: float) -> np.ndarray:
    # 12 neighbours: +-a_i and +-(a_i - a_j) in lattice coordinates
    k = 2 * np.pi * np.arange(L) / L
    k1, k2, k3 = np.meshgrid(k, k, k, indexing="ij")
    e = 2 * t * (np.cos(k1) + np.cos(k2) + np.cos(k3) + np.cos(k1 - k2) + np.cos(k1 - k3) + np.cos(k2 - k3))
    return e.reshape(-1)


def chain(L: int, t: float) -> np.ndarray:
    k = 2 * np.pi * np.arange(L) / L
    return 2 * t * np.cos(k)


CASES = {
    # name: (eigenvalues, a, M)
    "square_L16_t1": (square(16, 1.0), 4.05, 64),
    "honeycomb_L12_t-2.7": (honeycomb(12, -2.7), 8.2, 64),
    "fcc_L6_t1": (fcc(6, 1.0), 12.5, 48),
    "chain_L64_t1": (chain(64, 1.0), 2.5, 64),
}


def main() -> None:
    arrays = {}
    for name, (eps, a, M) in CASES.items():
        arrays[name] = cheb_trace(eps / a, M)
        arrays[name + "__a"] = np.array([a])
    np.savez(HERE / "exact_moments.npz", **arrays)
    counts = {
        # square 64x64 periodic, 1NN: 4 neighbours per site; rescale adds N diagonals
        "square_64x64_pbc": {"N": 4096, "nnz_H": 4 * 4096, "nnz_Ht": 5 * 4096},
        # honeycomb 1024x1024 periodic + on-site disorder: 3 neighbours + diagonal
        "honeycomb_1024x1024_pbc_disorder": {"N": 2097152, "nnz_H": 4 * 2097152, "nnz_Ht": 4 * 2097152},
        # square 256x256 open-x / periodic-y: 4N - 2*256 (no wrap in x)
        "square_256x256_openx_pbcy": {"N": 65536, "nnz_H": 4 * 65536 - 2 * 256, "nnz_Ht": 5 * 65536 - 2 * 256},
        # FCC 128^3 periodic + disorder: 12 neighbours + diagonal
        "fcc_128_pbc_disorder": {"N": 2097152, "nnz_H": 13 * 2097152, "nnz_Ht": 13 * 2097152},
    }
    (HERE / "counts.json").write_text(json.dumps(counts, indent=1) + "\n")


if __name__ == "__main__":
    main()
