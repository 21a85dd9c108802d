"""Occupied-bin plans of the single-vector fg! with G (sfh_models_set_occupied, onepass.cu)
against the FP64 oracle on the stored templates and against the dense kernel.

Hess diagrams leave most bins empty (the production workload fills about a fifth); with
G requested the kernel streams only the occupied bins' template rows and adds the empty
bins through the template column sums over them.  Tolerances as the dense FP32 tests:
|ΔlogL| <= 1e-6 per 1e4 stars, G within 2e-6 of Σ|M|(|w| + |1 - w|), w within 2e-6, and
the composite output exactly 1.0 in the empty bins (w = 1 - 0/max(c, eps), as fg!
leaves it)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _band(nbins, nt, seed, n_stars=1e5, occupied=0.25):
    """Templates with a populated band (a fraction `occupied` of the bins) and faint tails
    elsewhere, so that a Poisson draw leaves the tails empty."""
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt))
    band = rng.random(nbins) < occupied
    M[~band] *= 1e-9
    r = np.exp(rng.standard_normal(nt))
    r *= n_stars / (M @ r).sum()
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M), r, data


def _check(O, M, r, data, v, G, comp):
    Mst = M.astype(np.float32).astype(np.float64)
    v_ref, G_ref, w_ref = O.fg(r, Mst, data)
    assert abs(v - v_ref) <= 1e-6 * max(1.0, data.sum() / 1e4), (v, v_ref)
    scale = np.abs(Mst).T @ (np.abs(w_ref) + np.abs(1.0 - w_ref)) + 1e-300
    assert np.max(np.abs(G - G_ref) / scale) <= 2e-6
    np.testing.assert_allclose(comp, w_ref, rtol=2e-6, atol=2e-6)
    assert np.all(comp[data == 0] == 1.0)


def _fg(sfh, H, r, data):
    comp = np.empty(H.nbins)
    G = np.empty(H.nt)
    v = sfh.fg_(True, G, r, H, data, comp)
    return v, G, comp


VARIANTS = [(16, 1, "phased", 0), (32, 1, "phased", 0), (16, 2, "phased", 0),
            (16, 1, "skewed", 0), (32, 1, "phased", 1)]
SHAPES = [(37, 33), (1005, 65), (7500, 127), (152 * 32 * 3 + 5, 97), (60000, 1200)]


@pytest.mark.parametrize("bins,ctas,schedule,run", VARIANTS)
@pytest.mark.parametrize("nbins,nt", SHAPES)
def test_plan_matches_oracle(sfh, O, nbins, nt, bins, ctas, schedule, run):
    M, r, data = _band(nbins, nt, seed=3 * nbins + nt)
    H = sfh.Models(M, storage="f32")
    H.set_occupied("on")
    H.set_path("onepass")
    H.set_onepass_tile(bins)
    H.set_onepass_ctas(ctas)
    H.set_onepass_schedule(schedule)
    H.set_onepass_run(run)
    v, G, comp = _fg(sfh, H, r, data)
    nocc, sparse, _ = H.occupied_info()
    assert sparse and nocc == int(np.count_nonzero(data))
    _check(O, M, r, data, v, G, comp)
    v2, G2, comp2 = _fg(sfh, H, r, data)  # repeatable
    assert v2 == v and np.array_equal(G2, G) and np.array_equal(comp2, comp)


def test_plan_agrees_with_dense_kernel(sfh, O):
    M, r, data = _band(60000, 1200, seed=5, n_stars=1e6, occupied=0.22)
    H = sfh.Models(M, storage="f32")
    H.set_path("onepass")
    out = {}
    for mode in ("off", "auto"):
        H.set_occupied(mode)
        out[mode] = _fg(sfh, H, r, data)
    nocc, sparse, build_ms = H.occupied_info()
    assert sparse and 0 < nocc < 0.6 * M.shape[0] and build_ms > 0
    (v0, G0, c0), (v1, G1, c1) = out["off"], out["auto"]
    occ = data != 0
    assert np.all(c1[~occ] == 1.0) and np.all(c0[~occ] == 1.0)
    np.testing.assert_allclose(c1[occ], c0[occ], rtol=2e-7, atol=0)
    assert abs(v1 - v0) <= 1e-6 * data.sum() / 1e4
    Mst = M.astype(np.float32).astype(np.float64)
    scale = np.abs(Mst).T @ (np.abs(c0) + np.abs(1 - c0)) + 1e-300
    assert np.max(np.abs(G1 - G0) / scale) <= 2e-6
    _check(O, M, r, data, v1, G1, c1)


def test_auto_keeps_dense_diagrams_dense(sfh):
    rng = np.random.default_rng(1)
    M = np.asfortranarray(rng.random((7500, 50)))
    r = np.exp(rng.standard_normal(50))
    r *= 1e5 / (M @ r).sum()
    data = rng.poisson(M @ r).astype(float)  # every bin occupied
    H = sfh.Models(M, storage="f32")
    _fg(sfh, H, r, data)
    nocc, sparse, _ = H.occupied_info()
    assert nocc == 7500 and not sparse


def test_device_data_changed_in_place_is_folded_in_exactly(sfh, O):
    """Counts written into bins the plan holds as empty: the launch folds them in (same
    results as the oracle on the new data), flags the plan, and the next call builds a
    new one."""
    import torch
    M, r, data = _band(20000, 200, seed=9, n_stars=1e5)
    H = sfh.Models(M, storage="f32")
    H.set_occupied("on")
    ctx = H.ctx
    dev = torch.device("cuda", 0)
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_c = torch.empty(M.shape[0], dtype=torch.float64, device=dev)
    d_G = torch.empty(M.shape[1], dtype=torch.float64, device=dev)
    d_L = torch.empty(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    L = sfh.load()

    def call():
        rc = L.sfh_fg_dev(ctx.handle, H.handle, d_r.data_ptr(), d_n.data_ptr(), d_c.data_ptr(),
                          d_G.data_ptr(), d_L.data_ptr(), 2.220446049250313e-16)
        assert rc == 0
        ctx.synchronize()
        return d_L.item(), d_G.cpu().numpy(), d_c.cpu().numpy()

    v, G, comp = call()
    _check(O, M, r, data, v, G, comp)
    nocc0, sparse, _ = H.occupied_info(d_n.data_ptr())
    assert sparse and nocc0 == np.count_nonzero(data)
    # occupy 37 empty bins (spread over the CTAs' shares), empty 5 occupied ones
    rng = np.random.default_rng(2)
    empty = np.flatnonzero(data == 0)
    occ = np.flatnonzero(data != 0)
    new = data.copy()
    new[rng.choice(empty, 37, replace=False)] = rng.integers(1, 9, 37)
    new[rng.choice(occ, 5, replace=False)] = 0.0
    d_n.copy_(torch.tensor(new, device=dev))
    torch.cuda.synchronize()
    v, G, comp = call()  # the old plan: folded in
    _check(O, M, r, new, v, G, comp)
    assert H.occupied_info(d_n.data_ptr())[0] == nocc0  # not rebuilt yet
    v, G, comp = call()  # a new plan for the new counts
    _check(O, M, r, new, v, G, comp)
    assert H.occupied_info(d_n.data_ptr())[0] == np.count_nonzero(new)


def test_host_arrays_follow_the_data(sfh, O):
    """The host-array entry shares one plan slot per handle: new counts in the same or
    another array are checked and folded in, in either host-access mode."""
    from sfhgpu._lib import SFH_HOST_ACCESS_DIRECT, SFH_HOST_ACCESS_STAGED
    M, r, data = _band(20000, 200, seed=13, n_stars=1e5)
    H = sfh.Models(M, storage="f32")
    H.set_occupied("on")
    rng = np.random.default_rng(4)
    for mode in (SFH_HOST_ACCESS_STAGED, SFH_HOST_ACCESS_DIRECT):
        try:
            H.ctx.host_access = mode
        except sfh.SFHError:
            continue
        d = data.copy()
        for it in range(4):
            v, G, comp = _fg(sfh, H, r, d)
            _check(O, M, r, d, v, G, comp)
            d = d.copy() if it % 2 else d  # a new array, or the same one refilled
            z = np.flatnonzero(d == 0)
            d[rng.choice(z, 11, replace=False)] = 3.0
    H.ctx.host_access = -1


def test_fit_on_a_sparse_diagram_matches_the_dense_fit(sfh):
    """The device BFGS driver replays its evaluations from a captured graph: the plan is
    built by its eager first evaluation and used inside the graph."""
    M, r, data = _band(20000, 60, seed=17, n_stars=1e5)
    res = {}
    for mode in ("off", "on"):
        H = sfh.Models(M, storage="f32")
        H.set_occupied(mode)
        res[mode] = sfh.fit_templates(H, data, gtol=1e-6)
    f0, f1 = res["off"].mle.result.fun, res["on"].mle.result.fun
    assert abs(f1 - f0) <= 1e-6 * data.sum() / 1e4
    mu0, mu1, sg = res["off"].mle.mu, res["on"].mle.mu, res["off"].mle.sigma
    assert np.all(np.abs(mu1 - mu0) <= 1e-2 * sg + 1e-9 * np.max(mu0))
