"""The oracle of the self-energy contraction and convolution against known answers (CPU)."""
import numpy as np
import pytest

from oracle import selfc as osc


def test_mwm_identity_screening():
    # W = c·1: mwm[ω, p] = wkq·c_ω·Σ_I |M_pI|²
    rng = np.random.default_rng(1)
    nb1, nb2, N, nom = 3, 5, 17, 4
    M = rng.standard_normal((nb1, nb2, N)) + 1j * rng.standard_normal((nb1, nb2, N))
    c = rng.standard_normal(nom) + 0.3j * rng.standard_normal(nom)
    eps = np.zeros((N, N, nom), dtype=complex)
    for w in range(nom):
        eps[:, :, w] = c[w] * np.eye(N)
    wkq = 0.125
    out = osc.mwm_k(M, eps, wkq)
    want = wkq * c[:, None, None] * np.sum(np.abs(M) ** 2, axis=-1)[None]
    assert np.allclose(out, want, rtol=1e-13, atol=0)


def test_mwm_q0_terms():
    # only the pairs (r, ibgw + r + ncg_c) change, by the head/wing formula
    rng = np.random.default_rng(2)
    nb1, nb2, N, nom = 3, 8, 6, 2
    M = rng.standard_normal((nb1, nb2, N)) + 1j * rng.standard_normal((nb1, nb2, N))
    eps = rng.standard_normal((N, N, nom)) + 1j * rng.standard_normal((N, N, nom))
    head = rng.standard_normal(nom) + 1j * rng.standard_normal(nom)
    w1 = rng.standard_normal((N, nom)) + 1j * rng.standard_normal((N, nom))
    w2 = rng.standard_normal((N, nom)) + 1j * rng.standard_normal((N, nom))
    base = osc.mwm_k(M, eps, 0.5)
    q0 = osc.mwm_k(M, eps, 0.5, q0=(head, w1, w2, 0.7, 1.3, 2, 1))
    d = q0 - base
    for r in range(nb1):
        ie2 = 1 + r + 2
        for w in range(nom):
            want = 1.3 * head[w] + 0.7 * np.sum(M[r, ie2] * w2[:, w]) + 0.7 * np.sum(np.conj(M[r, ie2]) * w1[:, w])
            assert abs(d[w, r, ie2] - want) < 1e-12 * (1 + abs(want))
        d[:, r, ie2] = 0
    assert np.all(d == 0)


def _gl_mesh(n, wmax):
    x, wx = np.polynomial.legendre.leggauss(n)
    # Ω = wmax·((1+x)/2)², dense near 0 where f varies
    u = 0.5 * (1 + x)
    return wmax * u * u, wmax * u * wx


@pytest.mark.parametrize("e", [0.7, -1.3, 2.5])
def test_convolution_closed_form(e):
    # f(Ω) = 1/(Ω² + a²):  1/π ∫_0^∞ f(Ω)(e − iω)/((e − iω)² + Ω²) dΩ = 1/(2a(a·sign e + e − iω)),
    # checked at ω ≤ 10 where the cut-off at ω_max = 1e4 costs < 1e-9
    a = 0.8
    om, wom = _gl_mesh(1600, 1.0e4)
    f = 1.0 / (om ** 2 + a * a)
    for iom in np.nonzero(om <= 10.0)[0][::37]:
        sc = osc.fr_convolution2(e, f, f[iom], om, om[iom], wom)
        want = 1.0 / (2 * a * (a * np.sign(e) + e - 1j * om[iom]))
        assert abs(sc - want) / abs(want) < 1e-9


def test_convolution_constant_function_is_the_arctan_tail():
    # mwm constant in ω: the sum vanishes and only mwm/π·atan(ω_max/(e − iω)) is left
    om = np.geomspace(0.01, 50.0, 12)
    wom = np.gradient(om)
    mwm = np.full((12, 1, 1), 0.3 - 0.2j)
    sc = osc.all_fr_convolutions(np.array([-0.4]), mwm, om, wom)[0]
    want = (0.3 - 0.2j) / osc.PI_F * np.arctan(om[-1] / (-0.4 - 1j * om))
    assert np.allclose(sc, want, rtol=1e-14, atol=0)


def test_interp_convolution_reduces_to_plain_on_the_same_mesh():
    # with the dense mesh equal to the coarse one the spline is the identity
    pytest.importorskip("scipy")
    rng = np.random.default_rng(4)
    om = np.geomspace(0.02, 40.0, 10)
    wom = np.gradient(om)
    mwm = rng.standard_normal((10, 2, 3)) + 1j * rng.standard_normal((10, 2, 3))
    enk = rng.standard_normal(3)
    a = osc.interp_fr_convolutions(enk, mwm, om, om, wom)
    b = osc.all_fr_convolutions(enk, mwm, om, wom)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-14)


def test_svd_convolution_is_linear_in_the_basis():
    # mwm[l] = δ_{l,l0}·g: sc = Σ_ie2 g[ie2]·Cnl[l0, ie2]
    rng = np.random.default_rng(5)
    om = np.geomspace(0.02, 40.0, 8)
    wom = np.gradient(om)
    nl, nb1, nb2 = 3, 2, 4
    Ul = rng.standard_normal((nl, 8)) + 0j
    enk = rng.standard_normal(nb2)
    g = rng.standard_normal((nb1, nb2)) + 1j * rng.standard_normal((nb1, nb2))
    mwm = np.zeros((nl, nb1, nb2), dtype=complex)
    mwm[1] = g
    sc = osc.svd_fr_convolutions(enk, mwm, Ul, om, wom)
    cnl = osc.many_fr_convolutions(enk, Ul, om, wom)
    assert np.allclose(sc, g @ cnl[1], rtol=1e-13, atol=0)
    # a basis function convolved alone is fr_convolution2 of it
    want = osc.fr_convolution2(enk[2], Ul[0], Ul[0, 5], om, om[5], wom)
    assert cnl[0, 2, 5] == want


def test_spline_matrix_applies_the_reference_spline():
    """S·y is the cubic spline of y with the boundary conditions of
    mcommon.py:135 (second derivative 0 at the first point, slope 0 at the
    last, extrapolating), evaluated on the dense mesh — for any data y."""
    from scipy import interpolate

    from pygw_gb300.selfc import spline_matrix
    rng = np.random.default_rng(3)
    omega = np.sort(rng.uniform(0.01, 50.0, 24))
    dense = np.concatenate([np.linspace(0.005, 60.0, 200), omega])
    S = spline_matrix(omega, dense)
    assert S.shape == (dense.size, omega.size)
    y = rng.standard_normal((omega.size, 3))
    ref = interpolate.CubicSpline(omega, y, axis=0, bc_type=((2, np.zeros(3)), (1, np.zeros(3))),
                                  extrapolate=True)(dense)
    assert np.allclose(S @ y, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    # at the nodes the spline interpolates
    assert np.allclose(S[200:], np.eye(omega.size), atol=1e-12)


def test_selfc_k_chunk_fits_the_budget():
    """The self-energy's k-chunk and frequency batch keep the split-precision
    workspace within the budget (host arithmetic and size queries only)."""
    from pygw_gb300 import _lib
    from pygw_gb300.selfc import mixed_k_chunk
    lib = _lib.load()
    for P, npb, nom, budget in [(3200, 1200, 48, 64 << 30), (3200, 1200, 48, 8 << 30), (90, 128, 16, 1 << 30)]:
        nk, nb = mixed_k_chunk(P, npb, nom, budget=budget)
        assert nk >= 1 and 1 <= nb <= nom
        assert nb == 1 or lib.pg_selfc_mwm_workspace(nk, P, npb, nb, 1) <= budget
