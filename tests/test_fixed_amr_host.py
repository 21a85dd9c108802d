"""Host helpers of fixed_amr: construct_x0_mdf and truncate_relweights
(hierarchical/construct_x0_mdf.jl:58-71, fixed_amr.jl:225-243), the properties
fixed_amr_test.jl:24-58 checks."""
import numpy as np


def _grid():
    la = np.repeat(np.round(np.arange(8.0, 10.0 + 1e-9, 0.1), 10), 26)
    mh = np.tile(np.round(np.arange(-2.5, 0.0 + 1e-9, 0.1), 10), 21)
    return la, mh


def test_construct_x0_mdf_constant_sfr():
    from sfhgpu import construct_x0_mdf
    la, _ = _grid()
    rng = np.random.default_rng(1)
    sh = rng.permutation(la)  # input order does not matter
    x0 = construct_x0_mdf(sh, 13.7)
    uniq = list(dict.fromkeys(sh.tolist()))
    assert x0.size == len(uniq)
    srt = sorted(uniq) + [np.log10(13.7e9)]
    dt = np.diff(10.0 ** np.asarray(srt))
    sfr = [x0[i] / dt[srt.index(uniq[i])] for i in range(len(uniq))]
    assert np.allclose(sfr, sfr[0])
    assert np.isclose(construct_x0_mdf(la, 13.7).sum(), 1.0)
    assert np.isclose(construct_x0_mdf(la, 13.7, normalize_value=1e5).sum(), 1e5)


def test_truncate_relweights_matches_definition():
    from sfhgpu import LinearAMR, GaussianDispersion, calculate_coeffs, truncate_relweights
    la, mh = _grid()
    rw = calculate_coeffs(LinearAMR(0.05, -1.0 - 0.05 * 12.0), GaussianDispersion(0.2),
                          np.ones(21), la, mh)
    for u in np.unique(la):
        assert np.isclose(rw[la == u].sum(), 1.0)
    keep = []
    for u in dict.fromkeys(la.tolist()):
        good = np.nonzero(la == u)[0]
        keep += list(good[rw[good] >= 0.05 * rw[good].max()])
    assert list(truncate_relweights(0.05, rw, la)) == keep
    assert list(truncate_relweights(0.0, rw, la)) == list(range(la.size))
