"""CPU-only checks: the C-ABI library loads and exports every declared symbol, and
the host-side preprocessing mirrors agree with the oracle."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    with open(os.path.join(ROOT, "include", "sfhgpu.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sfh_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    import ctypes
    import sfhgpu
    from sfhgpu import _lib
    L = sfhgpu.load()
    decl = _declared_symbols()
    assert decl, "no declarations parsed"
    for name in decl:
        assert hasattr(L, name), f"{name} declared in include/sfhgpu.h but not exported"
    assert sorted(_lib.EXPORTED) == decl
    assert L.sfh_abi_version() == 1
    assert L.sfh_status_string(2) == b"shape mismatch"
    # no compute without a GPU: only argument validation, which never touches CUDA
    assert L.sfh_ctx_create(0, None) == 1  # SFH_ERR_ARG
    del ctypes


def test_entry_points_reject_missing_arguments_without_a_gpu():
    """Argument validation runs before any CUDA call: a NULL context or output is
    SFH_ERR_ARG (1) for the hard-binning, mock-observation and fit entry points."""
    import ctypes as C
    import sfhgpu
    from sfhgpu._lib import FitOptions, FitResult
    L = sfhgpu.load()
    n = C.c_int64()
    assert L.sfh_bin_cmd(None, None, None, None, 0, None, 1, None, 1, None) == 1
    assert L.sfh_bin_cmd_dev(None, None, None, None, 0, None, 1, None, 1, None) == 1
    assert L.sfh_model_cmd(None, None, None, None, None, 0, 1, 0, None, None, C.byref(n)) == 1
    assert L.sfh_model_cmd_dev(None, None, None, None, None, 0, 1, 0, None, None, C.byref(n)) == 1
    opt, res = FitOptions(), FitResult()
    assert L.sfh_fit_bfgs(None, None, None, None, C.byref(opt), None, None, C.byref(res)) == 1
    assert L.sfh_fit_bfgs_dev(None, None, None, None, C.byref(opt), None, None, C.byref(res)) == 1
    assert L.sfh_models_set_onepass_run(None, None, 4) == 1
    assert L.sfh_models_set_onepass_schedule(None, None, 1) == 1


def test_host_mini_spacing_and_interpolation_match_oracle(O):
    from sfhgpu import synthetic as S
    from sfhgpu import templates as T
    for la, mh in ((6.6, -2.0), (8.3, -1.0), (10.1, 0.3)):
        m, mags = S.isochrone(la, mh)
        colors = mags[0] - mags[1]
        for dmag in (0.0125, 0.04):
            a, sa = T.mini_spacing(m, colors, mags[1], dmag, True)
            b, sb = O.mini_spacing(m, colors, mags[1], dmag)
            assert np.array_equal(a, b)
            np.testing.assert_array_equal(sa, sb)
            np.testing.assert_array_equal(T.interpolate_mini(m, mags[0], a),
                                          O.interpolate_mini(m, mags[0], a))
    np.testing.assert_array_equal(T.midpoints([1.0, 2.0, 2.2, 2.1]), O.midpoints([1.0, 2.0, 2.2, 2.1]))


def test_duplicate_knots_follow_sort_ingested(O):
    # PARSEC isochrones repeat masses (data/isochrone.txt has one); sort_ingested nudges
    # the repeat to nextfloat (src/simulate.jl:54-63).
    from sfhgpu import templates as T
    m = np.array([0.1, 0.2, 0.2, 0.3])
    v = np.array([10.0, 9.0, 8.0, 7.0])
    q = np.array([0.1, 0.15, 0.2, 0.25, 0.3])
    np.testing.assert_array_equal(T.interpolate_mini(m, v, q), O.interpolate_mini(m, v, q))


def test_imf_weights_match_oracle(O):
    from sfhgpu import templates as T
    imf = T.Kroupa2001()
    oimf = O.kroupa2001()
    assert imf.mean() == pytest.approx(O.imf_mean(oimf), rel=1e-13)
    ms = np.array([0.08, 0.1, 0.3, 0.49999, 0.5, 0.7, 1.5, 100.0, 120.0])
    np.testing.assert_allclose(imf(ms), [O.imf_pdf(oimf, x) for x in ms], rtol=1e-13)
    mini = np.linspace(0.1, 1.5, 50)
    c = np.linspace(1, 0.5, 50)
    np.testing.assert_allclose(T.calculate_weights(mini, c, imf, 1e3, imf.mean()),
                               O.calculate_weights(mini, c, oimf, 1e3, imf.mean()), rtol=1e-13)


def test_construct_x0_reference_values():
    # test/fitting/fitting_core_test.jl:196-212
    from sfhgpu.fitting import construct_x0
    r = construct_x0(np.tile([1.0, 2.0, 3.0], 3), 1e-5, normalize_value=5)
    np.testing.assert_allclose(r, np.tile([0.015015015015015015, 0.15015015015015015,
                                           1.5015015015015016], 3), rtol=1e-7)
    assert r.sum() == pytest.approx(5, rel=1e-7)


def test_stack_models_layout():
    from sfhgpu.fitting import stack_models
    A = np.array([[0, 0, 0], [1, 1, 1], [0, 0, 0]], float)
    B = np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], float)
    np.testing.assert_array_equal(stack_models([A, B]),
                                  np.array([[0, 1, 0, 0, 1, 0, 0, 1, 0],
                                            [0, 0, 1, 0, 0, 1, 0, 0, 1]], float).T)


def test_synthetic_is_deterministic():
    from sfhgpu import synthetic as S
    w = S.config2()
    assert w.ntempl == 1200 and w.grid == (200, 300)
    a = S.isochrone_batch(S.small())
    b = S.isochrone_batch(S.small())
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(S.coefficients(5, 1), S.coefficients(5, 1))
