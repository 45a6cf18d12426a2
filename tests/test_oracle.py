"""Pins the CPU oracle (no GPU): analytic known answers, golden fixtures,
scipy cross-checks and the reference's own FFT/DCT algorithm restated in numpy."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.fft
import scipy.sparse as sp

import oracle as orc
from helpers import landau_gauge, rel_err, spec_from, with_onsite_zeros

GOLD = Path(__file__).resolve().parent / "golden"


def _csc(spec):
    cp, ri, v = orc.build_csc(spec)
    n = len(cp) - 1
    return n, cp, ri, v


def test_random_phase_kets_unit_modulus_and_seeded(tb):
    k = orc.random_phase_kets(100, 3, 7)
    assert np.allclose(np.abs(k), 1 / np.sqrt(100), rtol=0, atol=1e-15)
    # same generator in the library's host helper: bit-identical
    k2 = tb.bases_of_uniform_ampl_with_random_phases(100, 3, 7)
    assert np.array_equal(k, k2)
    assert not np.array_equal(k, orc.random_phase_kets(100, 3, 8))


def test_uniform_disorder_matches_formula():
    M = (1 << 64) - 1

    def mix(x):
        x = (x + 0x9E3779B97F4A7C15) & M
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M
        return x ^ (x >> 31)

    def u01(seed, stream, idx):
        k = mix(seed ^ mix((stream + 0x632BE59BD9B4E019) & M))
        h = mix((k + idx * 0xD1B54A32D192ED03) & M)
        return (h >> 11) * 2.0 ** -53

    v = orc.uniform_disorder(50, 0.8, 3)
    ref = np.array([0.8 * (u01(3, 0xD150D3D, i) - 0.5) for i in range(50)])
    assert np.array_equal(v, ref)
    assert np.all(np.abs(v) <= 0.4)


@pytest.mark.parametrize("model,atoms,maxnn", [("Square", ["A"], 3), ("Honeycomb", ["A", "B"], 3),
                                               ("Kagome", ["A", "B", "C"], 2), ("Lieb", ["A", "B", "C"], 2),
                                               ("FCC", ["A"], 2), ("Cubic", ["A"], 3), ("Chain", ["A"], 3)])
def test_nn_shells_oracle_vs_library(tb, model, atoms, maxnn):
    cell = getattr(tb, model)()
    bases, pos = cell.geometry()
    for ai, a in enumerate(atoms):
        for nn in range(1, maxnn + 1):
            to, lv = orc.nn_shell(cell.dim, bases, pos, ai, nn)
            # library: add this single shell to a fresh cell and read back the raw members
            c = getattr(tb, model)()
            c.add_hopping(a, nn, 1.0)
            f, t, v, _ = c.hoppings()
            # every oracle member appears in the library table directly or as its h.c.
            lib_set = {(int(x), int(y), tuple(int(q) for q in w)) for x, y, w in zip(f, t, v)}
            for b, w in zip(to, lv):
                h = (ai, int(b), tuple(int(q) for q in w))
                hc = (int(b), ai, tuple(-int(q) for q in w))
                assert h in lib_set or hc in lib_set, (model, a, nn, h)


def test_nn_shell_sizes():
    # square 1NN: 4 members; FCC 1NN: 12; honeycomb A 1NN: 3 B sites
    sq = orc.nn_shell(2, np.eye(3)[:, :2], np.zeros((1, 3)), 0, 1)[0]
    assert len(sq) == 4
    fb = np.array([[0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]).T
    assert len(orc.nn_shell(3, fb, np.zeros((1, 3)), 0, 1)[0]) == 12
    s3 = np.sqrt(3)
    hb = np.array([[1.5, -s3 / 2, 0], [1.5, s3 / 2, 0]]).T
    to, _ = orc.nn_shell(2, hb, np.array([[0, 0, 0], [1, 0, 0.0]]), 0, 1)
    assert sorted(to.tolist()) == [1, 1, 1]


def test_nnz_counts_square_c1(tb):
    cell = tb.Square().add_hopping("A", 1, 1.0)
    spec = spec_from(cell, (64, 64), mode=orc.MODE_PERIODIC_BARE, is_complex=False, extend=[1, 1])
    n, cp, ri, v = _csc(spec)
    counts = json.loads((GOLD / "counts.json").read_text())["square_64x64_pbc"]
    assert n == counts["N"] and len(ri) == counts["nnz_H"]
    ocp, ori, ov = orc.rescale_csc(n, cp, ri, v, 4.05, 0.0)
    assert len(ori) == counts["nnz_Ht"]
    # CSC invariants: sorted rows, symmetric pattern
    for j in range(n):
        assert np.all(np.diff(ri[cp[j]:cp[j + 1]]) > 0)
    M = sp.csc_matrix((v, ri, cp), shape=(n, n))
    assert abs(M - M.T).max() == 0


def test_nnz_counts_open_x_periodic_y(tb):
    cell = tb.Square().add_hopping("A", 1, 1.0)
    L = 32
    spec = spec_from(cell, (L, L), mode=orc.MODE_PERIODIC_BARE, is_complex=True, extend=[0, 1])
    n, cp, ri, v = _csc(spec)
    assert len(ri) == 4 * L * L - 2 * L


@pytest.mark.parametrize("name,model,span,nn_t", [("square_L16_t1", "Square", (16, 16), 1.0),
                                                  ("honeycomb_L12_t-2.7", "Honeycomb", (12, 12), -2.7),
                                                  ("fcc_L6_t1", "FCC", (6, 6, 6), 1.0),
                                                  ("chain_L64_t1", "Chain", (64,), 1.0)])
def test_oracle_exact_trace_golden(tb, name, model, span, nn_t):
    gold = np.load(GOLD / "exact_moments.npz")
    mu_exact, a = gold[name], float(gold[name + "__a"][0])
    cell = getattr(tb, model)().add_hopping("A", 1, nn_t)
    spec = spec_from(cell, span, mode=orc.MODE_PERIODIC_BARE, is_complex=False, extend=[1] * len(span))
    n, cp, ri, v = _csc(spec)
    ocp, ori, ov = orc.rescale_csc(n, cp, ri, v, a, 0.0)
    eye = np.asfortranarray(np.eye(n, dtype=np.complex128))
    mu = orc.cheb_moments(n, ocp, ori, ov, len(mu_exact), eye, eye)
    assert np.max(np.abs(mu - mu_exact)) / mu_exact[0] < 1e-12


def _scipy_moments(M, n_mom, bras, kets):
    T0 = kets.copy()
    T1 = M @ kets
    mu = [np.real(np.vdot(bras, T0)), np.real(np.vdot(bras, T1))]
    for _ in range(2, n_mom):
        T2 = 2 * (M @ T1) - T0
        mu.append(np.real(np.vdot(bras, T2)))
        T0, T1 = T1, T2
    return np.array(mu)


@pytest.mark.parametrize("cplx", [False, True])
def test_oracle_vs_scipy_recursion(tb, cplx):
    cell = with_onsite_zeros(tb.Honeycomb().add_hopping("A", 1, -2.7))
    span = (10, 9)
    N = 2 * 90
    V = orc.uniform_disorder(N, 1.0, 1)
    G, c = landau_gauge(2 * np.pi / 17)
    spec = spec_from(cell, span, mode=orc.MODE_SPARSE, is_complex=cplx, scalar_site=V,
                     gauge_linear=np.concatenate([G.reshape(-1), c]) if cplx else None)
    n, cp, ri, v = _csc(spec)
    a, b = 9.0, 0.1
    ocp, ori, ov = orc.rescale_csc(n, cp, ri, v, a, b)
    M = sp.csc_matrix((ov, ori, ocp), shape=(n, n))
    assert abs(M - M.conj().T).max() < 1e-15   # Hermitian
    kets = orc.random_phase_kets(n, 5, 11)
    bras = orc.random_phase_kets(n, 5, 12)
    for br in (kets, bras):
        mu = orc.cheb_moments(n, ocp, ori, ov, 40, br, kets)
        ref = _scipy_moments(M, 40, br, kets)
        assert rel_err(mu, ref) < 1e-12


def test_oracle_moments_errors_and_limits():
    cp = np.array([0, 1], dtype=np.int32)
    ri = np.array([0], dtype=np.int32)
    v = np.array([0.5])
    k = np.ones((1, 1), dtype=np.complex128, order="F")
    with pytest.raises(ValueError):
        orc.cheb_moments(1, cp, ri, v, 1, k, k)
    mu = orc.cheb_moments(1, cp, ri, v, 6, k, k)
    assert np.allclose(mu, np.cos(np.arange(6) * np.arccos(0.5)))


def test_doubling_identity_in_oracle(tb):
    cell = tb.Square().add_hopping("A", 1, 1.0)
    spec = spec_from(cell, (12, 12), mode=orc.MODE_PERIODIC_BARE, is_complex=False, extend=[1, 1])
    n, cp, ri, v = _csc(spec)
    ocp, ori, ov = orc.rescale_csc(n, cp, ri, v, 4.05, 0.0)
    kets = orc.random_phase_kets(n, 4, 0)
    mu = orc.cheb_moments(n, ocp, ori, ov, 32, kets, kets)
    blocks = orc.cheb_blocks(n, ocp, ori, ov, 16, kets)
    for k in range(1, 16):
        vv = np.real(np.vdot(blocks[k], blocks[k]))
        assert abs(2 * vv - mu[0] - mu[2 * k]) < 1e-12 * mu[0]
        if k < 15:
            vw = np.real(np.vdot(blocks[k + 1], blocks[k]))
            assert abs(2 * vw - mu[1] - mu[2 * k + 1]) < 1e-12 * mu[0]


def test_rescale_semantics():
    # 3x3 with one missing diagonal and an explicit zero
    d = sp.csc_matrix(np.array([[1.0, 2.0, 0], [2.0, 0, 0], [0, 0, 5.0]]))
    d.sort_indices()
    cp, ri, v = d.indptr.astype(np.int32), d.indices.astype(np.int32), d.data.copy()
    ocp, ori, ov = orc.rescale_csc(3, cp, ri, v, 2.0, 1.0)
    M = sp.csc_matrix((ov, ori, ocp), shape=(3, 3)).toarray()
    assert np.array_equal(M, (np.array([[1.0, 2.0, 0], [2.0, 0, 0], [0, 0, 5.0]]) - np.eye(3)) / 2.0)
    assert len(ori) == 5   # 4 entries of H plus (1,1) from the identity


def test_commutator_zero_diagonal(tb):
    cell = with_onsite_zeros(tb.Square().add_hopping("A", 1, 1.0))
    spec = spec_from(cell, (5, 4), mode=orc.MODE_SPARSE, is_complex=False, scalar_site=np.zeros(20))
    n, cp, ri, v = _csc(spec)
    x = orc.position_diag(spec, 0)
    cv = orc.commutator_values(n, cp, ri, v, x)
    for j in range(n):
        for p in range(cp[j], cp[j + 1]):
            i = ri[p]
            assert cv[p] == x[i] * v[p] - v[p] * x[j]
            if i == j:
                assert cv[p] == 0.0


def test_kernels_against_formulas():
    N = 37
    n = np.arange(N)
    g = orc.kernel_seq(orc.K_JACKSON, N)
    N1 = N + 1
    ref = ((N1 - n) * np.cos(np.pi * n / N1) + np.sin(np.pi * n / N1) / np.tan(np.pi / N1)) / N1
    assert np.allclose(g, ref, rtol=1e-14, atol=1e-15) and abs(g[0] - 1) < 1e-14
    assert np.allclose(orc.kernel_seq(orc.K_LORENTZ, N, 4.0), np.sinh(4 * (1 - n / N)) / np.sinh(4.0), rtol=1e-14)
    assert np.allclose(orc.kernel_seq(orc.K_FEJER, N), 1 - n / N)
    assert np.all(orc.kernel_seq(orc.K_DIRICHLET, N) == 1.0)
    assert np.allclose(orc.kernel_seq(orc.K_WANG_ZUNGER, N, 2.0, 3.0), np.exp(-(n * 2.0 / N) ** 3))


def test_resolvent_coefficients_closed_form():
    # inside the band: Im alpha_0 = -1/sin th, Im alpha_n = -2 cos(n th)/sin th
    e = 0.3
    al = np.zeros(2 * 20)
    orc.lib().tbo_expn_coef_alpha_seq(e, 0.0, 20, al.ctypes.data)
    th = np.arccos(e)
    ref = -2 * np.cos(np.arange(20) * th) / np.sin(th)
    ref[0] = -1 / np.sin(th)
    assert np.allclose(al[1::2], ref, rtol=1e-12)


def _ref_radix_fft_conj(x, start, step, n, N, select=0):
    """numpy restatement of numerical::fft::radix_fft_conj (TB/numerical.h:198-231)."""
    xN = len(x)

    def s(i):
        j = start + i * step
        return j + N if j < 0 else j

    def add_sub(i, j):
        if i < xN and j < xN:
            return x[i] + x[j], x[i] - x[j]
        if j >= xN:
            return x[i], x[i]
        return x[j], -x[j]

    if n <= 1:
        return [x[s(0)]]
    if n == 2:
        return list(add_sub(s(0), s(1)))
    if n == 4:
        a, b = add_sub(s(0), s(2))
        c, d = add_sub(s(1), s(3))
        if select > 0:
            return [a + c, b + 1j * d]
        return [a + c, b + 1j * d, a - c, b - 1j * d]
    U = _ref_radix_fft_conj(x, start, 2 * step, n // 2, N)
    Z = _ref_radix_fft_conj(x, start + step, 4 * step, n // 4, N)
    Z_ = _ref_radix_fft_conj(x, start - step, 4 * step, n // 4, N)
    X = [0j] * (n // 2 if select > 0 else n)
    for i in range(n // 4):
        om = np.exp(-2j * np.pi * i / n)
        wZ = Z[i] * np.conj(om)
        wZ_ = Z_[i] * om
        wZc = wZ + wZ_
        wZc_ = -1j * (wZ - wZ_)
        X[i] = U[i] + wZc
        X[i + n // 4] = U[i + n // 4] - wZc_
        if select > 0:
            continue
        X[i + n // 2] = U[i] - wZc
        X[i + 3 * n // 4] = U[i + n // 4] + wZc_
    return X


def _ref_dct_iii_complex(C):
    """numpy restatement of numerical::fft::dct_iii_complex (TB/numerical.h:233-255)."""
    N = len(C)
    Z = [0j] * N
    Z[0] = C[0]
    for i in range(1, N // 2):
        om = np.exp(-2j * np.pi * i / (4 * N))
        Z[i] = np.conj(om) * (C[i] - 1j * C[N - i])
        Z[N - i] = om * (C[i] + 1j * C[N - i])
    Z[N // 2] = np.sqrt(2) * C[N // 2]
    y = _ref_radix_fft_conj(Z, 0, 1, N, N)
    x = [0j] * N
    for i in range(N // 2):
        x[2 * i] = y[i]
        x[2 * i + 1] = y[N - i - 1]
    return np.array(x)


@pytest.mark.parametrize("N", [8, 16, 64])
def test_reference_dct_iii_is_redft01(N):
    rng = np.random.default_rng(N)
    C = rng.normal(size=N) + 1j * rng.normal(size=N)
    k = np.arange(N)
    direct = np.array([C[0] + 2 * np.sum(C[1:] * np.cos(np.pi * np.arange(1, N) * (kk + 0.5) / N)) for kk in k])
    assert np.allclose(_ref_dct_iii_complex(list(C)), direct, rtol=1e-12, atol=1e-12)
    # and the half-length conj FFT: phi[k] = sum_n C_n exp(+i pi n k / N), first N outputs of length 2N
    half = _ref_radix_fft_conj(list(C), 0, 1, 2 * N, 2 * N, 1)
    direct_h = np.array([np.sum(C * np.exp(1j * np.pi * np.arange(N) * kk / N)) for kk in k])
    assert np.allclose(half, direct_h, rtol=1e-12, atol=1e-12)


def test_oracle_fft_is_scipy_dct3():
    rng = np.random.default_rng(1)
    mu = rng.normal(size=64)
    g = orc.kernel_seq(orc.K_JACKSON, 64)
    E, val = orc.green_imag_fft(g, mu)
    y = scipy.fft.dct(g * mu, type=3, norm=None)   # REDFT01 (unnormalised)
    assert np.allclose(val, y / np.sqrt(1 - E ** 2), rtol=1e-12, atol=1e-12)
    assert np.allclose(E, np.cos((np.arange(64) + 0.5) * np.pi / 64))


def test_dos_integrates_to_one(tb):
    # rho(e) = sum (2-d_n0) g_n mu_n T_n(e) / (pi R sqrt(1-e^2)), mu_0 = R
    gold = np.load(GOLD / "exact_moments.npz")
    mu = gold["square_L16_t1"] / 256.0
    g = orc.kernel_seq(orc.K_JACKSON, len(mu))
    th = (np.arange(4000) + 0.5) * np.pi / 4000
    e = np.cos(th)
    f = orc.green_imag_eval(g, mu, e)
    rho = -f / np.pi
    integral = np.sum(rho * np.sin(th)) * (np.pi / 4000)   # de = sin th dth
    assert abs(integral - 1.0) < 1e-9
    assert np.allclose(rho, rho[::-1], atol=1e-12)      # bipartite: rho(e) = rho(-e)


def test_mu_nm_and_bastin_reduce_to_direct_sums():
    rng = np.random.default_rng(3)
    M, K = 6, 40
    L = rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))
    R = rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))
    mu = orc.mu_nm(L, R)
    assert np.allclose(mu, L.conj() @ R.T, rtol=1e-13)
    eps = np.array([-0.5, 0.1, 0.7])
    z = orc.bastin_zeta(mu, eps, 2.0)
    ref = []
    for x in eps:
        th, s = np.arccos(x), np.sqrt(1 - x * x)
        acc = 0
        for m in range(M):
            for n in range(M):
                am, an = (1 if m == 0 else 2), (1 if n == 0 else 2)
                G = am * an * ((x - 1j * n * s) * np.exp(1j * n * th) * np.cos(m * th)
                               + (x + 1j * m * s) * np.exp(-1j * m * th) * np.cos(n * th))
                acc += mu[m, n] * G
        ref.append(acc / (1 - x * x) ** 2 / 2.0)
    assert np.allclose(z, ref, rtol=1e-12)
