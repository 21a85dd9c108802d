"""Binary-star templates (RandomBinaryPairs): the oracle's restatement of binary_hess and of
partial_cmd_smooth's single/binary mix (src/StarFormationHistories.jl:627-706, 829-910),
pinned by the reference's doctests and tests for the pieces it uses and by invariants:

* mag2flux / flux2mag doctests (src/utilities.jl:52-55, 62-65);
* binary model fractions (test/cmd_simulation_test.jl:83-94);
* trapz (Trapz.jl) exact on piecewise-linear data;
* a binary fraction of 0 returns the single-star template;
* the binary template holds the summed pair weights (mass conservation of the smoothing
  inside a grid that contains every pair), whose closed form is
  prefac ((Σ a)^2 - Σ a^2) / 2 with a_i = ΔM_i (imf_i + imf_i+1)."""
import numpy as np
import pytest


def test_flux_doctests(O):
    assert O.mag2flux(15.0 - 25.0) == pytest.approx(10 ** (4 * (25.0 - 15.0) / 10))
    assert O.flux2mag(10000.0) + 25.0 == pytest.approx(25.0 - 5 * np.log10(10000.0) / 2)


def test_binary_model_fractions(sfh):
    assert sfh.NoBinaries().binary_system_fraction() == 0
    assert sfh.NoBinaries().binary_mass_fraction(None) == 0
    rb = sfh.RandomBinaryPairs(0.4)
    assert rb.binary_system_fraction() == 0.4
    assert rb.binary_mass_fraction(None) == pytest.approx(2 * 0.4 / 1.4)
    with pytest.raises(ValueError):
        sfh.RandomBinaryPairs(1.5)


def test_trapz(O, sfh):
    x = np.array([0.0, 0.5, 2.0, 3.0])
    y = 3.0 * x + 1.0
    assert O.trapz(x, y) == pytest.approx(1.5 * 9.0 + 3.0)
    rng = np.random.default_rng(1)
    x = np.sort(rng.random(50))
    y = rng.random(50)
    assert O.trapz(x, y) == pytest.approx(sfh.trapz(x, y), rel=1e-14)


def _iso(n=60):
    from sfhgpu import synthetic as S
    m, mags = S.isochrone(9.5, -1.0, n)
    return m, np.asarray(mags, dtype=np.float64)


def _models(O):
    from sfhgpu import synthetic as S
    E = [O.ErrModel(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    Cm = [O.ComplModel(c.A, c.m50, c.rho) for c in S.completeness_models()]
    return E, Cm


def test_zero_fraction_is_single(O):
    m, mags = _iso()
    E, Cm = _models(O)
    imf = O.kroupa2001()
    ex, ey = (-0.6, 0.06, 50), (19.0, 0.22, 50)
    single = O.partial_cmd_smooth(m, mags, E, Cm, 1, (0, 1), imf, 25.0, 1.0, O.imf_mean(imf), ex, ey)
    mixed = O.partial_cmd_smooth_binary(m, mags, E, Cm, 1, (0, 1), imf, 25.0, 1.0, O.imf_mean(imf),
                                        0.0, ex, ey)
    np.testing.assert_array_equal(single, mixed)


def test_binary_mass_conservation(O):
    m, mags = _iso(40)
    E, Cm = _models(O)
    # constant photometric error 0.2 (exponent 0, capped): stamps resolved by the grid, so
    # the covariant kernel's 3-point Gauss-Legendre rule (:303-304) keeps their mass
    E = [O.ErrModel(np.e, 0.0, 0.0, 0.0, 0.2) for _ in E]
    Cm = [O.ComplModel(1.0, 1e9, 1.0) for _ in Cm]  # completeness 1
    imf = O.kroupa2001()
    mm = O.imf_mean(imf)
    # a grid that holds every pair's colour and magnitude and their smoothing windows
    ex, ey = (-1.0, 0.05, 80), (-3.0, 0.1, 200)
    H = O.binary_hess(m, mags, E, Cm, 1, (0, 1), imf, 1.0, mm, ex, ey)
    iv = np.array([O.imf_pdf(imf, v) for v in m])
    a = np.diff(m) * (iv[:-1] + iv[1:])
    pscale = O.trapz(m, iv)
    prefac = 1.0 / mm / 4.0 / pscale
    # pairs (i, j > i) over the n - 1 intervals; the last interval pairs with none
    tot = prefac * (a.sum() ** 2 - (a ** 2).sum()) / 2.0
    assert H.sum() == pytest.approx(tot, rel=1e-5)


def test_binary_needs_y_in_colors(O):
    m, mags = _iso(30)
    E, Cm = _models(O)
    imf = O.kroupa2001()
    with pytest.raises(ValueError):
        O.binary_hess(m, mags, E, Cm, 2, (0, 1), imf, 1.0, O.imf_mean(imf), (-0.6, 0.06, 50),
                      (19.0, 0.22, 50))
