"""mu_nm GEMM: tcgen05 split-TF32 path and CUDA-core path vs an FP64 reference
on the same complex64-rounded blocks.  Stated bound for random blocks (where
mu is far smaller than the sum of its terms): max|err| <= 5e-6 * max|mu|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _blocks(M, K, seed):
    rng = np.random.default_rng(seed)
    L = (rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))) / np.sqrt(K)
    R = (rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))) / np.sqrt(K)
    return L, R


def _ref(L, R):
    L32 = L.astype(np.complex64).astype(np.complex128)
    R32 = R.astype(np.complex64).astype(np.complex128)
    return L32.conj() @ R32.T


@pytest.mark.parametrize("M,K", [(128, 512), (40, 3001), (200, 20000), (256, 70000)])
@pytest.mark.parametrize("tensor", [False, True])
def test_mu_gemm(gpu, M, K, tensor):
    tb = gpu
    L, R = _blocks(M, K, M + K)
    mu = tb.mu_from_blocks(L, R, tensor=tensor)
    ref = _ref(L, R)
    err = np.max(np.abs(mu - ref)) / np.max(np.abs(ref))
    assert err <= 5e-6, err
