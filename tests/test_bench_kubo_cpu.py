"""bench.py's CPU baseline of the reference's Kubo path on a small periodic
square lattice (no GPU): the recursion and velocity product are the oracle's
serial C walk, the contraction rate comes from a complex128 GEMM, and the
extrapolated solve time is 2 M steps + (M + 1) products + M^2 N R
multiply-adds at the measured rates."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


class _Csc:
    """Stands in for a device matrix: to_csc() gives the host CSC arrays."""

    def __init__(self, A):
        self.A = A

    def to_csc(self):
        return (self.A.indptr.astype(np.int32), self.A.indices.astype(np.int32), self.A.data.astype(np.float64))


def _square(L):
    sp = pytest.importorskip("scipy.sparse")
    rows, cols = [], []
    for i in range(L):
        for j in range(L):
            for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                rows.append(i * L + j)
                cols.append(((i + di) % L) * L + (j + dj) % L)
    return sp.csc_matrix((np.full(len(rows), 0.25), (rows, cols)), shape=(L * L, L * L))


def test_kubo_cpu_baseline_extrapolation():
    sys.path.insert(0, str(ROOT))
    import bench

    A = _square(48)
    M, R, steps = 96, 4, 6
    out = bench.kubo_cpu_baseline(_Csc(A), _Csc(A), M, R, steps)
    rec, gemm = out["recursion"], out["gemm"]
    assert out["kind"] == "port" and rec["cores"] == 1 and rec["steps_timed"] == steps
    assert rec["s_per_step"] > 0 and rec["operator_product_s"] > 0 and gemm["complex_macs_per_s"] > 0
    n = A.shape[0]
    assert gemm["macs"] == M * M * n * R
    assert out["recursion_s"] == pytest.approx(2 * M * rec["s_per_step"] + (M + 1) * rec["operator_product_s"])
    assert out["gemm_s"] == pytest.approx(M * M * n * R / gemm["complex_macs_per_s"])
    assert out["value_s"] == pytest.approx(out["recursion_s"] + out["gemm_s"])
