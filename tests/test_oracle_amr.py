"""LinearAMR hierarchical objective (amr.jl): the oracle's analytic gradient against
central finite differences, the host model against the oracle, and the constraint
constructor (the amr.jl:222-226 doctest)."""
import numpy as np


def _amr_problem(O, seed=3, nages=4, nmh=5, nb=300):
    rng = np.random.default_rng(seed)
    la = np.repeat(np.linspace(10.0, 8.5, nages), nmh)
    mh = np.tile(np.linspace(-2.5, 0.0, nmh), nages)
    M = rng.random((nb, nages * nmh))
    v = np.concatenate([rng.random(nages) * 1e3 + 100, [0.1, -2.0, 0.3]])
    data = rng.poisson(M @ np.full(nages * nmh, 50.0)).astype(float)
    return la, mh, M, v, data


def test_oracle_amr_gradient_matches_finite_differences(O):
    la, mh, M, v, data = _amr_problem(O)
    f, G = O.amr_fg(v, 13.7, M, data, la, mh)
    h = np.maximum(np.abs(v) * 1e-6, 1e-7)
    fd = np.array([(O.amr_fg(v + hh * e, 13.7, M, data, la, mh, want_g=False)[0]
                    - O.amr_fg(v - hh * e, 13.7, M, data, la, mh, want_g=False)[0]) / (2 * hh)
                   for e, hh in zip(np.eye(v.size), h)])
    assert np.all(np.abs(G - fd) <= 1e-6 * np.maximum(np.abs(fd), 1e-3))
    # fixed parameters keep a zero gradient entry
    _, Gf = O.amr_fg(v, 13.7, M, data, la, mh, free=(False, True, False))
    assert Gf[-3] == 0.0 and Gf[-1] == 0.0 and Gf[-2] == G[-2]


def test_host_linear_amr_matches_oracle(O):
    from sfhgpu.sampling import GaussianDispersion, LinearAMR, calculate_coeffs
    la, mh, M, v, data = _amr_problem(O, seed=4)
    amr = LinearAMR(v[-3], v[-2], 13.7)
    assert amr(9.5) == O.linear_amr(v[-3], v[-2], 13.7, 9.5)
    coeffs = calculate_coeffs(amr, GaussianDispersion(v[-1]), v[:-3], la, mh)
    c = M @ coeffs
    ref = -O.amr_fg(v, 13.7, M, data, la, mh, want_g=False)[0]
    logL = np.sum(np.where(data > 0, data - c - data * np.log(np.where(data > 0, data, 1) / c), -c))
    assert abs(logL - ref) <= 1e-9 * abs(ref)


def test_linear_amr_from_constraints():
    from sfhgpu.sampling import LinearAMR
    a = LinearAMR.from_constraints((-2.5, 13.7), (-1.0, 0.0), 13.7)
    b = LinearAMR.from_constraints((-1.0, 0.0), (-2.5, 13.7), 13.7)
    assert (a.alpha, a.beta) == (b.alpha, b.beta)
    assert np.isclose(a(np.log10(13.7e9)), -2.5) and np.isclose(a(np.log10(1.0)), -1.0, atol=1e-9)


def test_oracle_log_amr_gradient_and_mh_from_z(O):
    from sfhgpu.sampling import MH_from_Z, dMH_dZ
    rng = np.random.default_rng(5)
    nages, nmh, nb = 4, 5, 300
    la = np.repeat(np.linspace(10.0, 8.5, nages), nmh)
    mh = np.tile(MH_from_Z(10 ** np.linspace(-4, -2, nmh)), nages)
    M = rng.random((nb, nages * nmh))
    v = np.concatenate([rng.random(nages) * 1e3 + 100, [1e-4, 5e-5, 0.3]])
    data = rng.poisson(M @ np.full(nages * nmh, 50.0)).astype(float)
    f, G = O.amr_fg(v, 13.7, M, data, la, mh, kind=1)
    h = np.maximum(np.abs(v) * 1e-6, 1e-12)
    fd = np.array([(O.amr_fg(v + hh * e, 13.7, M, data, la, mh, want_g=False, kind=1)[0]
                    - O.amr_fg(v - hh * e, 13.7, M, data, la, mh, want_g=False, kind=1)[0])
                   / (2 * hh) for e, hh in zip(np.eye(v.size), h)])
    assert np.all(np.abs(G - fd) <= 1e-5 * np.maximum(np.abs(fd), 1e-3))
    for Z in (1e-4, 1e-3, 0.01524, 0.03):
        assert np.isclose(MH_from_Z(Z), O.mh_from_z(Z), rtol=1e-14, atol=1e-15)
        assert np.isclose(dMH_dZ(Z), O.dmh_dz(Z), rtol=1e-14)
    assert abs(MH_from_Z(0.01524)) < 1e-15  # [M/H] = 0 at the solar Z
