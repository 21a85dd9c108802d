"""The oracle against the reference's own known answers (CPU only).

Pins: test/fitting/fitting_core_test.jl:9-195, doctests of
src/StarFormationHistories.jl:55-75 / :485-500, dispersion_models.jl:63-67,
mzr.jl:245-249, and the properties of test/templates/template_test.jl:10-33.
"""
import numpy as np
import pytest


def _models3():
    return [np.array([[1, 1, 1], [0, 0, 0], [0, 0, 0]], float),
            np.array([[0, 0, 0], [1, 1, 1], [0, 0, 0]], float),
            np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], float)]


def _flat(models):
    return np.stack([m.ravel(order="F") for m in models], 1)


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_composite(O, T):
    A = np.array([[0, 0, 0], [1, 1, 1], [0, 0, 0]], T)
    B = np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], T)
    C = O.composite(_flat([A, B]), np.array([1, 2], T))
    assert np.array_equal(C, np.array([0, 1, 2, 0, 1, 2, 0, 1, 2], float))


@pytest.mark.parametrize("T,ri", [(np.float32, 0), (np.float64, 1)])
def test_loglikelihood(O, kats, T, ri):
    rtol = kats["rtol_float32_float64"]["value"][ri]
    C = np.array([[1, 1, 1], [2, 2, 2], [3, 3, 3]], T).astype(float)
    data = np.array([[1, 1, 1], [2, 2, 2], [2, 2, 2]], float)
    eps = O.eps_of(T)
    assert O.loglikelihood(C, data, eps) == pytest.approx(kats["loglikelihood"]["value"], rel=rtol)
    Cz = np.array([[1.5] * 3, [3] * 3, [3] * 3])
    dz = np.array([[0] * 3, [2] * 3, [2] * 3], float)
    assert O.loglikelihood(Cz, dz, eps) == pytest.approx(kats["loglikelihood_zero_data"]["value"],
                                                         rel=rtol)
    # 3-argument form through composite
    A = np.array([[1, 1, 1], [0, 0, 0], [0, 0, 0]], float)
    B = np.array([[0, 0, 0], [1, 1, 1], [1.5, 1.5, 1.5]], float)
    c = O.composite(_flat([A, B]), np.array([1, 2.0]))
    assert O.loglikelihood(c, data.ravel(order="F"), eps) == pytest.approx(
        kats["loglikelihood"]["value"], rel=rtol)


def test_loglikelihood_zero_sum_is_minus_inf(O):
    # loglikelihood returns -typemax(T) when the sum is exactly zero, fitting_base.jl:95
    assert O.loglikelihood(np.ones(4), np.ones(4)) == -np.inf


def test_gradients(O):
    C = np.array([[1, 1, 1], [2, 2, 2], [3, 3, 3]], float)
    data = np.array([[1, 1, 1], [2, 2, 2], [2, 2, 2]], float)
    model = np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], float)
    assert O.grad_single(model, C, data) == pytest.approx(-1.0, rel=1e-12)
    Cz = np.array([[1.5] * 3, [3] * 3, [3] * 3])
    dz = np.array([[0] * 3, [2] * 3, [2] * 3], float)
    assert O.grad_single(np.array([[1, 1, 1], [0, 0, 0], [0, 0, 0]], float), Cz, dz) == \
        pytest.approx(-3.0, rel=1e-12)
    M = _flat(_models3())
    c = O.composite(M, np.array([1.5, 3, 3]))
    G, w = O.grad_inplace(c, M, data.ravel(order="F"))
    np.testing.assert_allclose(G, [-1, -1, -1], rtol=1e-12)
    np.testing.assert_allclose(w, 1 - data.ravel(order="F") / c)  # composite overwritten
    G, _ = O.grad_inplace(c, M, dz.ravel(order="F"))
    np.testing.assert_allclose(G, [-3, -1, -1], rtol=1e-12)


def test_fg(O, kats):
    M = _flat(_models3())
    data = np.array([[1, 1, 1], [2, 2, 2], [2, 2, 2]], float).ravel(order="F")
    v, G, _ = O.fg(np.array([1.5, 3, 3]), M, data)
    assert -v == pytest.approx(kats["fg_negative"]["value"], rel=1e-12)
    np.testing.assert_allclose(-G, [-1, -1, -1], rtol=1e-12)
    v2, G2, _ = O.fg(np.array([1.5, 3, 3]), M, data, want_g=False)
    assert v2 == v and G2 is None


def test_interpolate_mini_doctest(O, kats):
    m_ini = [0.08, 0.10, 0.12, 0.14, 0.16]
    mags = [13.545, 12.899, 12.355, 11.459, 10.947]
    new = np.arange(0.08, 0.16 + 1e-12, 0.01)
    np.testing.assert_allclose(O.interpolate_mini(m_ini, mags, new),
                               kats["interpolate_mini_doctest"]["value"], rtol=1e-12)


def test_histogram_pix_doctest(O):
    assert O.histogram_pix(0.5, 0.0, 0.1) == pytest.approx(6)
    assert O.histogram_pix(0.55, 0.0, 0.1) == pytest.approx(6.5)
    assert O.histogram_pix(0.5, 1.0, -0.1) == pytest.approx(6)


def test_mini_spacing_properties(O, kats):
    # test/templates/template_test.jl:10-24
    m, sp = O.mini_spacing([0.08, 0.10, 0.12, 0.14, 0.16], [1.0, 0.99, 0.98, 0.97, 0.96],
                           [13.545, 12.899, 12.355, 11.459, 10.947], 0.1)
    assert len(m) > 5
    assert np.max(np.diff(m)) < kats["template_test_mini_spacing_max_diff"]["value"]
    np.testing.assert_allclose(sp, np.diff(m))


def test_midpoints(O):
    # test/templates/template_test.jl:26-33
    np.testing.assert_allclose(O.midpoints([1.0, 2.0, 2.2, 2.1]), [1.5, 2.1, 2.15])
    np.testing.assert_allclose(O.midpoints(np.arange(0.5, 1.0001, 0.1)), np.arange(0.55, 0.96, 0.1))


def test_dispersion_and_mzr_doctests(O, kats):
    L = O.lib()
    assert L.sfho_gauss_disp(0.2, 1.0, 1.2) == pytest.approx(np.exp(-0.5))
    A = L.sfho_gauss_disp(0.2, 1.0, 1.2)
    # gradient(GaussianDispersion(0.2), 1.0, 1.2) = (A (x-μ)²/σ³, A (x-μ)/σ²)
    g = kats["gaussian_dispersion_gradient"]["value"]
    assert A * (1.0 - 1.2) ** 2 / 0.2 ** 3 == pytest.approx(g)
    assert A * (1.0 - 1.2) / 0.2 ** 2 == pytest.approx(-g)
    assert L.sfho_powerlaw_mzr(1.0, -1.0, 6.0, 1e7) == pytest.approx(0.0, abs=1e-14)


def test_kernels_nonzero_three_cases(O):
    # test/templates/kernel_test.jl:1-43 (each configuration produces non-zero bins)
    sig = 0.1
    for cov, yc, sx in ((-1, 20.0, 0.1), (1, 19.0, 0.1), (0, 18.0, np.hypot(0.1, 0.1))):
        xc = 1.0
        xe = np.arange(xc - 5 * sig, xc + 5 * sig + 1e-9, sig / 10)
        ye = np.arange(yc - 5 * sig, yc + 5 * sig + 1e-9, sig / 10)
        nx, ny = len(xe) - 1, len(ye) - 1
        H = O.bin_cmd_smooth([xc], [yc], [sx], [sig], [1.0], cov, (xe[0], sig / 10, nx),
                             (ye[0], sig / 10, ny))
        assert np.any(H != 0)


def test_stamp_mass_conservation(O):
    # A stamp well inside the grid integrates to its weight (±5σ windows hold ~1 - 6e-7).
    H = O.bin_cmd_smooth([0.0], [0.0], [0.05], [0.05], [2.0], 0, (-1.0, 0.01, 200),
                         (-1.0, 0.01, 200))
    assert H.sum() == pytest.approx(2.0, rel=1e-5)
    H = O.bin_cmd_smooth([0.0], [0.0], [0.05], [0.05], [2.0], 1, (-1.0, 0.01, 200),
                         (-1.0, 0.01, 200))
    assert H.sum() == pytest.approx(2.0, rel=1e-4)


def _mzr_problem(seed=7, nages=6, nmh=5, nbins=400):
    rng = np.random.default_rng(seed)
    la = np.repeat(np.linspace(10.0, 8.0, nages), nmh)
    mh = np.tile(np.linspace(-2.5, 0.0, nmh), nages)
    M = rng.random((nbins, nages * nmh)) / 1e2
    R = rng.random(nages) * 1e4 + 1e3
    return la, mh, M, R


def test_mzr_coeffs_sum_to_stellar_mass(O):
    la, mh, M, R = _mzr_problem()
    c = O.mzr_calculate_coeffs(1.0, -1.0, 6.0, 0.2, R, la, mh)
    np.testing.assert_allclose(c.reshape(len(R), -1).sum(1), R, rtol=1e-12)


def test_mzr_gradient_matches_finite_differences(O):
    # The reference pins its analytic gradient with ForwardDiff (mzr_test.jl:76-113);
    # the FP64 oracle is pinned by central differences instead.
    la, mh, M, R = _mzr_problem()
    c = O.mzr_calculate_coeffs(0.5, -1.0, 6.0, 0.2, R, la, mh)
    data = np.random.default_rng(3).poisson(M @ c).astype(float)
    v = np.concatenate([R, [0.5, -1.0, 0.2]])
    f0, G = O.mzr_fg(v, 6.0, M, data, la, mh)
    for i in range(v.size):
        h = 1e-6 * max(1.0, abs(v[i]))
        vp, vm = v.copy(), v.copy()
        vp[i] += h
        vm[i] -= h
        fd = (O.mzr_fg(vp, 6.0, M, data, la, mh, want_g=False)[0] -
              O.mzr_fg(vm, 6.0, M, data, la, mh, want_g=False)[0]) / (2 * h)
        assert G[i] == pytest.approx(fd, rel=1e-5, abs=1e-7)
