"""GPU parity of the batched tensor-core objective (sfh_fg_batched_dev) against the FP64
oracle on the stored FP32 templates and the exact FP64 coefficient vectors.

With logL requested the composite comes from the exact digit-plane kernel
(batched_exact.cu): |ΔlogL| <= 1e-6 per 1e4 stars, the hot-path tolerance.  The gradient
G = W M runs on BF16 hi/lo planes of W and M with FP32 accumulation: its error is bounded
by 1e-4 of sum_i |M_ij| |w_i|.  Gradient-only calls form W from the hi/lo composite
(three BF16 products, FP32 accumulation) under the same gradient bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 2.220446049250313e-16


def _problem(nbins, nt, B, seed, n_stars, spread=0.3):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > 0.3)
    r0 = np.exp(rng.standard_normal(nt))
    r0 *= n_stars / (M @ r0).sum()
    data = rng.poisson(M @ r0).astype(float)
    R = r0[None, :] * np.exp(spread * rng.standard_normal((B, nt)))
    return np.asfortranarray(M.astype(np.float32)), R, data


def _run(sfh, M32, R, data, want_l=True, want_g=True, H=None):
    import torch
    L = sfh.load()
    H = H or sfh.Models(M32, storage="bf16x2")
    ctx = H.ctx
    dev = torch.device("cuda", 0)
    B, nt = R.shape
    d_R = torch.tensor(R, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_L = torch.empty(B, dtype=torch.float64, device=dev) if want_l else None
    d_G = torch.empty((B, nt), dtype=torch.float32, device=dev) if want_g else None
    torch.cuda.synchronize()
    rc = L.sfh_fg_batched_dev(ctx.handle, H.handle, d_R.data_ptr(), B, d_n.data_ptr(),
                              d_L.data_ptr() if want_l else None,
                              d_G.data_ptr() if want_g else None, EPS)
    sfh._lib.check(rc, ctx.handle, "sfh_fg_batched_dev")
    ctx.synchronize()
    return (d_L.cpu().numpy() if want_l else None), (d_G.cpu().numpy() if want_g else None)


def _check(O, M32, R, data, negL, G, nchk=6):
    Ms = np.asfortranarray(M32.astype(np.float64))
    B = R.shape[0]
    check = np.linspace(0, B - 1, min(B, nchk)).astype(int)
    ref_L, ref_G = O.fg_batched(R[check], Ms, data, nthreads=4)
    nst = data.sum()
    dL = np.abs(negL[check] - ref_L)
    # the hot-path bar: 1e-6 per 1e4 stars against FP64 on the stored templates
    assert np.all(dL <= 1e-6 * max(1.0, nst / 1e4)), (dL, nst)
    if G is not None:
        for k, b in enumerate(check):
            w = 1.0 - data / np.maximum(Ms @ R[b], EPS)
            scale = np.abs(Ms).T @ np.abs(w) + 1e-300
            assert np.max(np.abs(G[b] - ref_G[k]) / scale) <= 1e-4
    return dL.max() / max(1.0, nst / 1e4)


@pytest.mark.parametrize("nbins,nt,B,nst", [(7500, 50, 128, 1e5), (20000, 300, 300, 1e4),
                                            (4099, 77, 5, 1e5), (60000, 64, 256, 1e5),
                                            (1000, 1, 33, 1e4)])
def test_batched_against_oracle(sfh, O, nbins, nt, B, nst):
    M32, R, data = _problem(nbins, nt, B, seed=nbins + nt + B, n_stars=nst)
    negL, G = _run(sfh, M32, R, data)
    _check(O, M32, R, data, negL, G)


def test_batched_production_shape(sfh, O):
    """60,000 bins x 1,200 templates x 256 vectors, 1e6 stars: the batched workload's
    matrix, at the hot-path tolerance."""
    M32, R, data = _problem(60000, 1200, 256, seed=17, n_stars=1e6)
    negL, G = _run(sfh, M32, R, data)
    _check(O, M32, R, data, negL, G, nchk=4)


def test_batched_wide_coefficient_range(sfh, O):
    """Coefficient vectors spanning ~1e5 within a vector (exp(2 N(0,1)) spread): the
    per-vector exponent leaves the small entries fewer digits, the bar still holds."""
    M32, R, data = _problem(20000, 200, 64, seed=23, n_stars=1e5, spread=2.0)
    negL, G = _run(sfh, M32, R, data)
    _check(O, M32, R, data, negL, G)


def test_batched_logl_only_and_grad_only(sfh, O):
    M32, R, data = _problem(5000, 40, 64, seed=3, n_stars=1e4)
    negL, _ = _run(sfh, M32, R, data, want_l=True, want_g=False)
    _, G = _run(sfh, M32, R, data, want_l=False, want_g=True)
    negL2, G2 = _run(sfh, M32, R, data)
    np.testing.assert_array_equal(negL, negL2)   # deterministic: fixed reduction order
    # gradient-only calls form W from the hi/lo composite: the same bound against the oracle
    _check(O, M32, R, data, negL2, G)
    _check(O, M32, R, data, negL2, G2)


def test_batched_requires_bf16_storage(sfh):
    import torch
    L = sfh.load()
    M32, R, data = _problem(1000, 8, 4, seed=1, n_stars=1e3)
    H = sfh.Models(M32, storage="f32")
    dev = torch.device("cuda", 0)
    d_R = torch.tensor(R, device=dev)
    d_n = torch.tensor(data, device=dev)
    torch.cuda.synchronize()
    assert L.sfh_fg_batched_dev(H.ctx.handle, H.handle, d_R.data_ptr(), 4, d_n.data_ptr(),
                                None, None, 2.2e-16) == 1


def _band(nbins, nt, B, seed, n_stars, occupied=0.25, spread=0.3):
    """A populated band (a fraction `occupied` of the bins) and faint tails, so that most
    bins of the Poisson draw stay empty, as in Hess diagrams."""
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt))
    M[rng.random(nbins) >= occupied] *= 1e-9
    r0 = np.exp(rng.standard_normal(nt))
    r0 *= n_stars / (M @ r0).sum()
    data = rng.poisson(M @ r0).astype(float)
    R = r0[None, :] * np.exp(spread * rng.standard_normal((B, nt)))
    return np.asfortranarray(M.astype(np.float32)), R, data


@pytest.mark.parametrize("nbins,nt,B,nst", [(20000, 300, 128, 1e5), (60000, 1200, 256, 1e6),
                                            (7503, 65, 37, 1e4)])
def test_batched_occupied_plan_matches_oracle_and_dense(sfh, O, nbins, nt, B, nst):
    """The occupied-bin plan (a derived handle of the occupied rows; the empty bins through
    FP64 column sums) against the oracle and the dense call."""
    M32, R, data = _band(nbins, nt, B, seed=nbins + B, n_stars=nst)
    H = sfh.Models(M32, storage="bf16x2")
    out = {}
    for mode in ("off", "on"):
        H.set_occupied(mode)
        out[mode] = _run(sfh, M32, R, data, H=H)
        _check(O, M32, R, data, *out[mode], nchk=4)
    (L0, G0), (L1, G1) = out["off"], out["on"]
    assert np.max(np.abs(L1 - L0)) <= 1e-6 * max(1.0, data.sum() / 1e4)
    Ms = M32.astype(np.float64)
    for b in (0, B - 1):
        w = 1.0 - data / np.maximum(Ms @ R[b], EPS)
        scale = np.abs(Ms).T @ np.abs(w) + 1e-300
        assert np.max(np.abs(G1[b] - G0[b]) / scale) <= 1e-4


def test_batched_occupied_plan_negative_coefficient(sfh, O):
    """A negative coefficient turns the split logL off (each c subtracted per bin); the
    parent's empty bins then enter through Σ_j R_bj E_j."""
    M32, R, data = _band(8000, 40, 16, seed=5, n_stars=1e4)
    R[3, 7] = -0.5 * abs(R[3, 7])
    H = sfh.Models(M32, storage="bf16x2")
    H.set_occupied("on")
    negL, G = _run(sfh, M32, R, data, H=H)
    Ms = np.asfortranarray(M32.astype(np.float64))
    ref_L, _ = O.fg_batched(R[[0, 3]], Ms, data, nthreads=4)
    assert np.all(np.abs(negL[[0, 3]] - ref_L) <= 1e-6 * max(1.0, data.sum() / 1e4))


def test_batched_occupied_plan_follows_new_counts(sfh, O):
    """Counts written into plan-empty bins: the call finds them, evaluates densely, and the
    next call builds a plan for the new diagram."""
    import torch
    L = sfh.load()
    M32, R, data = _band(20000, 100, 64, seed=29, n_stars=1e5)
    H = sfh.Models(M32, storage="bf16x2")
    H.set_occupied("on")
    dev = torch.device("cuda", 0)
    d_R = torch.tensor(R, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_L = torch.empty(R.shape[0], dtype=torch.float64, device=dev)
    d_G = torch.empty(R.shape, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def call():
        rc = L.sfh_fg_batched_dev(H.ctx.handle, H.handle, d_R.data_ptr(), R.shape[0],
                                  d_n.data_ptr(), d_L.data_ptr(), d_G.data_ptr(), EPS)
        sfh._lib.check(rc, H.ctx.handle, "sfh_fg_batched_dev")
        H.ctx.synchronize()
        return d_L.cpu().numpy(), d_G.cpu().numpy()

    _check(O, M32, R, data, *call())
    nocc0 = H.occupied_info(d_n.data_ptr())[0]
    assert nocc0 == np.count_nonzero(data)
    rng = np.random.default_rng(3)
    new = data.copy()
    new[rng.choice(np.flatnonzero(data == 0), 23, replace=False)] = 4.0
    d_n.copy_(torch.tensor(new, device=dev))
    torch.cuda.synchronize()
    _check(O, M32, R, new, *call())
    _check(O, M32, R, new, *call())
    assert H.occupied_info(d_n.data_ptr())[0] == np.count_nonzero(new)
