"""The reference's cuSPARSE + cuBLAS moments algorithm, restated in
baseline/cusparse_kpm.cu as the timing baseline of the GPU path it replaces,
gives the oracle's moments (FP64, 1e-10 of mu_0) for both overloads."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu
LIB = Path(__file__).resolve().parent.parent / "baseline" / "_build" / "libref_cusparse.so"


def _fn(name):
    lib = C.CDLL(str(LIB))
    f = getattr(lib, name)
    f.restype = C.c_int
    f.argtypes = [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                  C.c_int32, C.c_void_p, C.c_void_p]
    return f


@pytest.mark.parametrize("cplx", [False, True])
def test_reference_gpu_algorithm_matches_oracle(gpu, cplx):
    tb = gpu
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (20, 18))
    X.set_scalar_disorder(1.0, 2)
    if cplx:
        G0 = np.zeros((3, 3))
        G0[1, 0] = 0.05
        X.set_gauge_linear(G0, np.zeros(3))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], complex if cplx else float)
    cp, ri, v = tb.GreenFunction(8, H, -8.7, 8.7).scaled_HE.to_csc()
    n, R, M = len(cp) - 1, 5, 40
    kets = np.asfortranarray(orc.random_phase_kets(n, R, 3))
    bras = np.asfortranarray(orc.random_phase_kets(n, R, 4))
    mu = np.zeros(M)
    t = np.zeros(2)
    v = np.ascontiguousarray(v)
    rc = _fn("ref_cusparse_braket_complex" if cplx else "ref_cusparse_braket_real")(
        n, len(ri), cp.ctypes.data, ri.ctypes.data, v.ctypes.data, M, bras.ctypes.data, kets.ctypes.data, R,
        mu.ctypes.data, t.ctypes.data)
    assert rc == 0
    ref = orc.cheb_moments(n, cp, ri, v, M, bras, kets)
    assert np.max(np.abs(mu - ref)) <= 1e-10 * abs(ref[0])
    assert t[0] >= t[1] > 0
