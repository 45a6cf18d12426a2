"""FP64 reconstruction on the device vs the oracle: kernels, resolvent sums,
the DCT-III (REDFT01) route and the DoS entry points."""
import math

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

KINDS = [(orc.K_DIRICHLET, 0, 0), (orc.K_FEJER, 0, 0), (orc.K_LORENTZ, 4.0, 0), (orc.K_JACKSON, 0, 0),
         (orc.K_LANCZOS, 3.0, 0), (orc.K_WANG_ZUNGER, 2.0, 3.0)]


@pytest.mark.parametrize("kind,p0,p1", KINDS)
def test_kernel_seq(gpu, kind, p0, p1):
    tb = gpu
    g = tb.Kernel(kind, p0, p1).seq(257)
    ref = orc.kernel_seq(kind, 257, p0, p1)
    assert np.allclose(g, ref, rtol=1e-13, atol=1e-15)


def _moments():
    rng = np.random.default_rng(0)
    n = 300
    mu = rng.normal(size=n) * np.exp(-np.arange(n) / 80.0)
    mu[0] = 4.0
    return mu


def test_green_imag_eval_and_dos(gpu):
    tb = gpu
    mu = _moments()
    g = orc.kernel_seq(orc.K_JACKSON, len(mu))
    z = np.concatenate([np.linspace(-0.99, 0.99, 101) + 0j, [0.3 + 0.01j, -0.2 - 0.05j, 1.3 + 0j]])
    zz = np.ascontiguousarray(np.stack([z.real, z.imag], 1))
    out = np.zeros(len(z))
    tb.capi.check(tb.capi.lib().tbk_green_imag_eval(len(mu), g.ctypes.data, mu.ctypes.data, len(z), zz.ctypes.data,
                                                   out.ctypes.data, None))
    ref = orc.green_imag_eval(g, mu, z)
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))
    e = np.linspace(-0.95, 0.95, 1024)
    rho = tb.dos_from_moments(mu, tb.Jackson(), 4.0, e)
    assert np.allclose(rho, -orc.green_imag_eval(g, mu, e) / 4.0 / math.pi, rtol=1e-12, atol=1e-14)


def test_green_fft(gpu):
    tb = gpu
    mu = _moments()
    g = orc.kernel_seq(orc.K_LORENTZ, len(mu), 4.0)
    for up in (1, 2):
        E = np.zeros(len(mu) * up)
        v = np.zeros(len(mu) * up)
        tb.capi.check(tb.capi.lib().tbk_green_imag_fft(len(mu), g.ctypes.data, mu.ctypes.data, up, E.ctypes.data,
                                                      v.ctypes.data, None))
        rE, rv = orc.green_imag_fft(g, mu, up)
        assert np.allclose(E, rE, rtol=0, atol=1e-15)
        assert np.max(np.abs(v - rv)) <= 1e-11 * np.max(np.abs(rv))


def test_density_of_states_seq_end_to_end(gpu):
    """TB/functions.h:15-32 on the 64x64 square lattice (complex Scalar), vs the
    oracle pipeline on the same seeded kets."""
    tb = gpu
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (64, 64))
    E = np.linspace(-0.9, 0.9, 256)
    dos = tb.density_of_states_seq(X, 256, E, -4.05, 4.05, complex, R=4, seed=0)
    # oracle pipeline
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], complex)
    cp, ri, v = H.to_csc()
    Emin, Emax = -4.05 - 1e-8, 4.05 + 1e-8
    a, b = (Emax - Emin) / 2, (Emax + Emin) / 2
    ocp, ori, ov = orc.rescale_csc(len(cp) - 1, cp, ri, v, a, b)
    kets = orc.random_phase_kets(4096, 4, 0)
    mu = orc.cheb_moments(4096, ocp, ori, ov, 256, kets, kets)
    g = orc.kernel_seq(orc.K_LORENTZ, 256, 4.0)
    ref = -orc.green_imag_eval(g, mu, E) / 4 / math.pi
    assert np.max(np.abs(dos - ref)) <= 1e-10 * np.max(np.abs(ref))


def test_density_of_states_function(gpu):
    tb = gpu
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (32, 32))
    H = X.get_Hamiltonian_sparse(complex)
    G = tb.GreenFunction(128, H, -4.001, 4.001)
    dos = tb.density_of_states_function(G, R=4, seed=1)
    E = np.linspace(-4.0, 4.0, 801)
    d = dos(E)
    # integral over E of rho(E) dE/a ~ 1 (rho is per rescaled energy)
    assert abs(float(np.sum((d[1:] + d[:-1]) * np.diff(E)) / 2) / G.a - 1.0) < 0.03
