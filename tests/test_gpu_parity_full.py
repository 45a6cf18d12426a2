"""Mixed-precision parity at the full size of the benchmark DoS.

Workload: honeycomb 1024 x 1024 periodic (2,097,152 sites), t = -2.7, on-site
disorder U[-0.5, 0.5] (seed 1), H~ = H / 8.7, M = 2048 moments, R = 32
random-phase vectors (seed 0), Chebyshev doubling, Jackson kernel, rho(E) on
4,096 Chebyshev nodes.

The complex64 recursion is compared over all 2048 moments with the complex128
(FP64) recursion of the same seeded vectors — the plain path that the smaller
tests pin to the CPU oracle at 1e-10 — and with the double-float recursion.

Stated bounds (the target: DoS within 1e-5 relative of the FP64 run):
  max_n |mu_n(mixed) - mu_n(fp64)| / mu_0            <= MU_TOL
  max_E |rho_mixed(E) - rho_fp64(E)| / max_E rho_fp64 <= RHO_TOL
  max_n |mu_n(dd) - mu_n(fp64)| / mu_0               <= 1e-10
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MU_TOL = 1e-5
RHO_TOL = 1e-5
L, T_HOP, W, BOUND, M, R, NE = 1024, -2.7, 1.0, 8.7, 2048, 32, 4096


@pytest.fixture(scope="module")
def config2(gpu):
    tb = gpu
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, T_HOP), (L, L))
    X.set_scalar_disorder(W, 1)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    G = tb.GreenFunction(M, H, -BOUND, BOUND)
    out = {}
    for prec in ("fp64", "mixed", "dd"):
        s = tb.KpmSolver(G.scaled_HE, R, precision=prec, doubling=True)
        out[prec] = s.run_random(M, 0)
        del s
    return tb, out


def test_config2_moments_all_2048(config2):
    tb, mu = config2
    ref = mu["fp64"]
    assert abs(ref[0] - R) < 1e-9
    err = np.abs(mu["mixed"] - ref) / ref[0]
    # error growth over n, reported in blocks of 256 moments
    blocks = [float(err[i:i + 256].max()) for i in range(0, M, 256)]
    print("mixed vs fp64, max |d mu_n| / mu_0 per 256 moments:", ["%.2e" % b for b in blocks])
    assert float(err.max()) <= MU_TOL, blocks
    assert float(np.max(np.abs(mu["dd"] - ref)) / ref[0]) <= 1e-10


def test_config2_rho_4096_energies(config2):
    tb, mu = config2
    E = np.cos((np.arange(NE) + 0.5) * np.pi / NE) * 0.999
    jack = tb.Jackson()
    rho_ref = tb.dos_from_moments(mu["fp64"], jack, R, E)
    rho_mix = tb.dos_from_moments(mu["mixed"], jack, R, E)
    rel = float(np.max(np.abs(rho_mix - rho_ref)) / np.max(rho_ref))
    print("max |d rho| / max rho = %.3e" % rel)
    assert rel <= RHO_TOL
    # the density integrates to one over the rescaled band (Chebyshev-Gauss nodes)
    c = 0.999
    w = np.pi / NE * c * np.sqrt(1.0 - (E / c) ** 2)          # dE of the nodes E = c cos(theta)
    assert abs(float(np.sum(rho_ref * w)) - 1.0) < 1e-3
