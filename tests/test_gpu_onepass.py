"""One-pass single-vector fg! (FP32 template storage, onepass.cu) against the FP64 oracle
on the stored templates and against the two-pass kernels.

Shapes exercise a tile with padding bins (nbins not a multiple of 32), a partial last
template box (nt not a multiple of 64), an odd number of 32-template groups, one template,
several tiles per CTA, and the 1,536-template limit.  Tolerances as the other FP32-storage
fg! tests: |ΔlogL| <= 1e-6 per 1e4 stars, G within 2e-6 of Σ|M|(|w| + |1 - w|), w within
2e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(nbins, nt, seed, n_stars=1e4, zero_frac=0.2):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > zero_frac)
    r = np.exp(rng.standard_normal(nt))
    r *= n_stars / (M @ r).sum()
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M), r, data


def _check(O, M, r, data, v, G, comp):
    Mst = M.astype(np.float32).astype(np.float64)
    v_ref, G_ref, w_ref = O.fg(r, Mst, data)
    assert abs(v - v_ref) <= 1e-6 * max(1.0, data.sum() / 1e4), (v, v_ref)
    # each bin's FP32-rounded composite moves w by about (n/c) 6e-8, so G's error scale is
    # Σ|M| (|w| + |1 - w|) (Σ|M||w| alone shrinks where the model fits the data)
    scale = np.abs(Mst).T @ (np.abs(w_ref) + np.abs(1.0 - w_ref)) + 1e-300
    assert np.max(np.abs(G - G_ref) / scale) <= 2e-6
    np.testing.assert_allclose(comp, w_ref, rtol=2e-6, atol=2e-6)


SHAPES = [(4, 1), (3, 2), (32, 32), (37, 33), (1004, 64), (1005, 65), (7500, 50), (7500, 127),
          (152 * 32 * 3 + 5, 97), (4868, 1536), (60000, 1200)]


# (tile bins, CTAs per SM, schedule, boxes per bulk copy; 0 = the default)
VARIANTS = [(16, 1, "phased", 0), (32, 1, "phased", 0), (16, 2, "phased", 0),
            (16, 1, "skewed", 0), (16, 1, "phased", 1), (16, 1, "phased", 2),
            (32, 1, "phased", 1), (16, 1, "skewed", 1)]


@pytest.mark.parametrize("bins,ctas,schedule,run", VARIANTS)
@pytest.mark.parametrize("nbins,nt", SHAPES)
def test_onepass_matches_oracle(sfh, O, nbins, nt, bins, ctas, schedule, run):
    M, r, data = _problem(nbins, nt, seed=7 * nbins + nt)
    H = sfh.Models(M, storage="f32")
    H.set_occupied("off")  # the dense kernel (test_gpu_occupied.py covers the plan)
    H.set_path("onepass")
    H.set_onepass_tile(bins)
    H.set_onepass_ctas(ctas)
    H.set_onepass_schedule(schedule)
    H.set_onepass_run(run)
    assert H.path == "onepass"
    vb, vc, vs, vr = H.onepass_variant
    assert vr in (1, 2, 4) and (run == 0 or vr <= run)
    comp = np.empty(nbins)
    G = np.empty(nt)
    v = sfh.fg_(True, G, r, H, data, comp)
    _check(O, M, r, data, v, G, comp)


def test_onepass_sparse_data_and_empty_bins(sfh, O):
    """Most bins empty (n = 0) and many zero composites (eps clamp): the case of sparse
    Hess diagrams."""
    M, r, data = _problem(20000, 200, seed=3, n_stars=300, zero_frac=0.9)
    M[:4000] = 0.0  # composite exactly 0 there: max(c, eps)
    data[:4000] = 0.0
    H = sfh.Models(M, storage="f32")
    H.set_path("onepass")
    comp = np.empty(M.shape[0])
    G = np.empty(M.shape[1])
    v = sfh.fg_(True, G, r, H, data, comp)
    _check(O, M, r, data, v, G, comp)


def test_onepass_agrees_with_twopass_and_is_deterministic(sfh):
    M, r, data = _problem(60000, 1200, seed=11, n_stars=1e6)
    H = sfh.Models(M, storage="f32")
    out = {}
    for path in ("onepass", "twopass", "onepass"):
        H.set_path(path)
        comp = np.empty(M.shape[0])
        G = np.empty(M.shape[1])
        v = sfh.fg_(True, G, r, H, data, comp)
        if path in out:  # second one-pass run: bitwise the same
            assert v == out[path][0]
            assert np.array_equal(G, out[path][1]) and np.array_equal(comp, out[path][2])
        out[path] = (v, G, comp)
    for run in (1, 2, 4):  # boxes per bulk copy: bitwise the same results
        H.set_path("onepass")
        H.set_onepass_run(run)
        comp = np.empty(M.shape[0])
        G = np.empty(M.shape[1])
        v = sfh.fg_(True, G, r, H, data, comp)
        assert v == out["onepass"][0] and np.array_equal(G, out["onepass"][1])
        assert np.array_equal(comp, out["onepass"][2])
    H.set_onepass_run(0)
    H.set_onepass_schedule("skewed")  # the skewed schedule: bitwise the phased one's
    comp = np.empty(M.shape[0])
    G = np.empty(M.shape[1])
    H.set_path("onepass")
    v = sfh.fg_(True, G, r, H, data, comp)
    assert v == out["onepass"][0] and np.array_equal(G, out["onepass"][1])
    assert np.array_equal(comp, out["onepass"][2])
    H.set_onepass_schedule("phased")
    H.set_onepass_tile(32)  # the other tile width: same results to rounding
    comp = np.empty(M.shape[0])
    G = np.empty(M.shape[1])
    v = sfh.fg_(True, G, r, H, data, comp)
    out["onepass32"] = (v, G, comp)
    v1, G1, c1 = out["onepass"]
    v2, G2, c2 = out["twopass"]
    v3, G3, c3 = out["onepass32"]
    assert abs(v1 - v2) <= 2e-5 * data.sum() / 1e4
    scale = np.abs(M.astype(np.float32).astype(np.float64)).T @ (np.abs(c2) + np.abs(1 - c2)) + 1e-300
    assert np.max(np.abs(G1 - G2) / scale) <= 4e-6
    np.testing.assert_allclose(c1, c2, rtol=4e-6, atol=4e-6)
    assert abs(v1 - v3) <= 2e-5 * data.sum() / 1e4
    assert np.max(np.abs(G1 - G3) / scale) <= 4e-6


def test_onepass_logl_only_and_composite_semantics(sfh, O):
    """Without G the call keeps the model in the composite (fg! with G === nothing)."""
    M, r, data = _problem(7500, 50, seed=5)
    H = sfh.Models(M, storage="f32")
    H.set_path("onepass")
    comp = np.empty(M.shape[0])
    v = sfh.fg_(True, None, r, H, data, comp)
    Mst = M.astype(np.float32).astype(np.float64)
    v_ref, _, _ = O.fg(r, Mst, data)
    assert abs(v - v_ref) <= 1e-6 * max(1.0, data.sum() / 1e4)
    np.testing.assert_allclose(comp, Mst @ r, rtol=2e-6)


def test_onepass_shape_limits(sfh):
    ok = sfh.Models(np.ones((4, 1536)), storage="f32")
    ok.set_path("onepass")
    assert ok.path == "onepass"
    H = sfh.Models(np.ones((4, 1537)), storage="f32")  # too many templates
    assert H.path == "twopass"  # auto
    with pytest.raises(Exception):
        H.set_path("onepass")
    odd = sfh.Models(np.ones((10, 5)), storage="f32")  # any bin count
    assert odd.path == "onepass"
    H64 = sfh.Models(np.ones((8, 4)), storage="f64")
    with pytest.raises(Exception):
        H64.set_path("onepass")


def test_autotune_reports_path(sfh, O):
    M, r, data = _problem(60000, 600, seed=13)
    H = sfh.Models(M, storage="f32")
    H.autotune(r, data, iters=3)
    assert H.path in ("onepass", "twopass")
    assert H.onepass_ms > 0
    comp = np.empty(M.shape[0])
    G = np.empty(M.shape[1])
    v = sfh.fg_(True, G, r, H, data, comp)
    _check(O, M, r, data, v, G, comp)
    H.ctx.synchronize()  # no timed-out wait was recorded
