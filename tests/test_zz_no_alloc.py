"""The no-allocation moments entry point (tbk_cheb_moments_noalloc) against the
regular drop-in entry point.

Callers that may not allocate device memory while they run (a process whose
HBM budget is already handed out, a host that lends device buffers but forbids
allocation) hand this entry point device buffers they already own; its work
space is a fixed array inside the library.  This file is collected last on
purpose: it must give the same moments as tbk_cheb_braket_real/complex (FP64
tolerance 1e-10 of mu_0) on two calls in a row, both in a fresh process and
after every other test, and the second call must leave the device's free
memory unchanged.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# (cells, R, M, complex): a ragged small case in both value types, the
# two-moment edge (only the first step's moments), a single vector, and a
# lattice whose N * R equals the scratch limit (1,048,576 entries)
CASES = [((24, 20), 6, 96, False), ((24, 20), 6, 96, True), ((16, 12), 3, 2, False), ((30, 18), 1, 40, True),
         ((256, 256), 8, 12, False)]


@pytest.mark.parametrize("cells,R,M,cplx", CASES)
def test_noalloc_matches_dropin_twice(gpu, cells, R, M, cplx):
    torch = pytest.importorskip("torch")
    tb = gpu
    from tight_binding_gb300 import capi

    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), cells)
    X.set_scalar_disorder(1.0, 3)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], complex if cplx else float)
    G = tb.GreenFunction(8, H, -8.7, 8.7)
    Mcsc = G.scaled_HE.to_scipy()
    n = Mcsc.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, R, 11)
    bras = tb.bases_of_uniform_ampl_with_random_phases(n, R, 12)
    ref = tb.Cheb_first_kind_seq_braket(Mcsc, M, bras, kets, precision="fp64")

    csr = Mcsc.tocsr()
    csr.sort_indices()
    rp = _device(torch, csr.indptr.astype(np.int32))
    ci = _device(torch, csr.indices.astype(np.int32))
    vals = csr.data.astype(np.complex128) if cplx else csr.data.astype(np.float64)
    vv = _device(torch, vals.view(np.float64))
    kd = _device(torch, kets.T)            # (R, N) row-major == N x R column-major
    bd = _device(torch, bras.T)
    outs = [torch.full((M,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
    st = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    for k, mu in enumerate(outs):
        free0 = torch.cuda.mem_get_info()[0]
        capi.check(capi.lib().tbk_cheb_moments_noalloc(n, rp.data_ptr(), ci.data_ptr(), vv.data_ptr(), int(cplx), M,
                                                      bd.data_ptr(), kd.data_ptr(), R, mu.data_ptr(), st))
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        if k == 1:     # the first call of a process may load the module and reserve the array
            assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
        got = mu.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 1e-10 * abs(ref[0]) + 1e-12


def test_noalloc_rejects_oversize(gpu):
    from tight_binding_gb300 import capi

    n, R = 1 << 18, 8          # N * R = 2,097,152 > 1,048,576
    rc = capi.lib().tbk_cheb_moments_noalloc(n, None, None, None, 0, 16, None, None, R, None, None)
    assert rc == capi.TBK_ERR_INVALID
    assert b"exceeds" in capi.lib().tbk_last_error()
