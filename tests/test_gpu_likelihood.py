"""GPU parity for composite! / loglikelihood / ∇loglikelihood! / fg! (C ABI) against
the FP64 oracle.  Tolerances: FP64 template storage rtol 1e-10; FP32 storage is
compared with the oracle evaluated on the same stored (FP32-rounded) templates."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _models3():
    return [np.array([[1, 1, 1], [0, 0, 0], [0, 0, 0]], float),
            np.array([[0, 0, 0], [1, 1, 1], [0, 0, 0]], float),
            np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], float)]


@pytest.mark.parametrize("T,ri", [(np.float32, 0), (np.float64, 1)])
def test_reference_kats(sfh, kats, T, ri):
    rtol = kats["rtol_float32_float64"]["value"][ri]
    C = np.array([[1, 1, 1], [2, 2, 2], [3, 3, 3]], T)
    data = np.array([[1, 1, 1], [2, 2, 2], [2, 2, 2]], np.int64)
    v = sfh.loglikelihood(C, data)
    assert v == pytest.approx(kats["loglikelihood"]["value"], rel=rtol)
    assert isinstance(v, T)
    Cz = np.array([[1.5] * 3, [3] * 3, [3] * 3], T)
    dz = np.array([[0] * 3, [2] * 3, [2] * 3], np.int64)
    assert sfh.loglikelihood(Cz, dz) == pytest.approx(kats["loglikelihood_zero_data"]["value"],
                                                      rel=rtol)
    models = [m.astype(T) for m in _models3()]
    M = sfh.stack_models(models)
    coeffs = np.array([1.5, 3, 3], T)
    # composite! flat form
    A = np.array([[0, 0, 0], [1, 1, 1], [0, 0, 0]], T)
    B = np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], T)
    C2 = np.zeros(9, T)
    sfh.composite_(C2, np.array([1, 2], T), sfh.stack_models([A, B]))
    assert np.array_equal(C2, np.array([0, 1, 2, 0, 1, 2, 0, 1, 2], T))
    # ∇loglikelihood! with data and with zeros in data
    for d, want in ((data, [-1, -1, -1]), (dz, [-3, -1, -1])):
        c = M @ coeffs
        G = np.empty(3, T)
        sfh.grad_loglikelihood_(G, c, M, d.ravel(order="F"))
        np.testing.assert_allclose(G, want, rtol=rtol)
        np.testing.assert_allclose(c, 1 - d.ravel(order="F") / (M @ coeffs), rtol=rtol)
    # single-model ∇loglikelihood
    g1 = sfh.grad_loglikelihood(np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], T), C, data)
    assert g1 == pytest.approx(-1, rel=rtol)
    # fg! with and without G
    comp = np.empty(9, T)
    G = np.empty(3, T)
    r = sfh.fg_(True, G, coeffs, M, data.ravel(order="F"), comp)
    assert -r == pytest.approx(kats["fg_negative"]["value"], rel=rtol)
    np.testing.assert_allclose(-G, [-1, -1, -1], rtol=rtol)
    r2 = sfh.fg_(True, None, coeffs, M, data.ravel(order="F"), comp)
    assert -r2 == pytest.approx(kats["fg_negative"]["value"], rel=rtol)
    np.testing.assert_allclose(comp, M @ coeffs, rtol=rtol)  # G === nothing: composite kept


def test_zero_sum_is_minus_inf(sfh):
    # Every term n - c - n log(n/c) is exactly 0 when n == c == 1, so the sum is 0 and the
    # reference returns -typemax(T) = -Inf (fitting_base.jl:95).  Zero composites are
    # clamped to eps and do not sum to zero.
    assert sfh.loglikelihood(np.ones(5), np.ones(5)) == -np.inf
    assert sfh.loglikelihood(np.zeros(5), np.zeros(5)) == pytest.approx(-5 * np.finfo(float).eps)


def _problem(nbins, nt, seed, n_stars=1e4, zero_frac=0.2):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > zero_frac)
    r = np.exp(rng.standard_normal(nt))
    m = M @ r
    r *= n_stars / m.sum()
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M), r, data


@pytest.mark.parametrize("nbins,nt", [(7500, 50), (7501, 37), (1003, 1), (64, 300), (60000, 24)])
@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_fg_against_oracle(sfh, O, nbins, nt, storage):
    M, r, data = _problem(nbins, nt, seed=nbins + nt)
    Mst = M.astype(np.float32).astype(np.float64) if storage == "f32" else M
    H = sfh.Models(M, storage=storage)
    comp = np.empty(nbins)
    G = np.empty(nt)
    v = sfh.fg_(True, G, r, H, data, comp)
    v_ref, G_ref, w_ref = O.fg(r, Mst, data)
    m_ref = O.composite(Mst, r)
    # composite (recomputed without G so the composite is kept)
    comp2 = np.empty(nbins)
    sfh.composite_(comp2, r, H)
    rt = 1e-10 if storage == "f64" else 2e-6
    np.testing.assert_allclose(comp2, m_ref, rtol=rt, atol=1e-300)
    np.testing.assert_allclose(comp, w_ref, rtol=rt, atol=rt)
    # logL: deviation per 1e4 stars
    nst = data.sum()
    tol = (1e-9 if storage == "f64" else 1e-6) * max(1.0, nst / 1e4)
    assert abs(v - v_ref) <= tol, (v, v_ref)
    # gradient: relative to the natural scale sum_i |M_ij w_i|
    scale = np.abs(Mst).T @ np.abs(w_ref) + 1e-300
    assert np.max(np.abs(G - G_ref) / scale) <= (1e-11 if storage == "f64" else 2e-6)


def test_fg_device_arrays_and_determinism(sfh, O):
    import torch
    M, r, data = _problem(20000, 200, seed=5, n_stars=1e6)
    H = sfh.Models(M, storage="f32")
    ctx = H.ctx
    dev = torch.device("cuda", 0)
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_c = torch.empty(M.shape[0], dtype=torch.float64, device=dev)
    d_G = torch.empty(M.shape[1], dtype=torch.float64, device=dev)
    d_L = torch.empty(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    L = sfh.load()
    outs = []
    for _ in range(3):
        rc = L.sfh_fg_dev(ctx.handle, H.handle, d_r.data_ptr(), d_n.data_ptr(), d_c.data_ptr(),
                          d_G.data_ptr(), d_L.data_ptr(), 2.220446049250313e-16)
        assert rc == 0
        ctx.synchronize()
        outs.append((d_L.item(), d_G.cpu().numpy().copy()))
    # bitwise deterministic (no atomics in the reduction order)
    assert all(o[0] == outs[0][0] and np.array_equal(o[1], outs[0][1]) for o in outs)
    v_ref, G_ref, _ = O.fg(r, M.astype(np.float32).astype(np.float64), data)
    assert abs(outs[0][0] - v_ref) <= 1e-6 * data.sum() / 1e4


@pytest.mark.parametrize("storage", ["f32", "f64"])
def test_fg_host_access_modes_are_bit_identical(sfh, O, storage):
    """sfh_fg through the mapped pinned staging and with the kernels on the caller's own
    arrays (where the device reads pageable host memory) give the same bits."""
    from sfhgpu._lib import SFH_HOST_ACCESS_DIRECT, SFH_HOST_ACCESS_STAGED
    M, r, data = _problem(20000, 200, seed=11, n_stars=1e6)
    H = sfh.Models(M, storage=storage)
    ctx = H.ctx
    res = {}
    for mode in (SFH_HOST_ACCESS_STAGED, SFH_HOST_ACCESS_DIRECT):
        try:
            ctx.host_access = mode
        except sfh.SFHError:
            pytest.skip("the device does not read pageable host memory directly")
        assert ctx.host_access == mode
        comp, G = np.empty(M.shape[0]), np.empty(M.shape[1])
        v = sfh.fg_(True, G, r, H, data, comp)
        v2 = sfh.fg_(True, G.copy(), r, H, data, comp.copy())  # repeatable
        res[mode] = (v, G, comp)
        assert v2 == v
    ctx.host_access = -1
    (v0, G0, c0), (v1, G1, c1) = res[SFH_HOST_ACCESS_STAGED], res[SFH_HOST_ACCESS_DIRECT]
    assert v0 == v1 and np.array_equal(G0, G1) and np.array_equal(c0, c1)
    Mst = M.astype(np.float32).astype(np.float64) if storage == "f32" else M
    v_ref, G_ref, _ = O.fg(r, Mst, data)
    assert abs(v1 - v_ref) <= 1e-6 * data.sum() / 1e4


def test_fg_array_layouts_and_repeated_calls_agree(sfh):
    """fg! on float64 flat arrays (the direct C call), on a C-ordered Hess matrix and a
    float32 composite (converted copies), and 300 calls in a row (each waiting on the
    context's completion word) all give the same bits."""
    M, r, data = _problem(20000, 200, seed=12, n_stars=1e6)
    H = sfh.Models(M, storage="f32")
    nb, nt = M.shape
    comp, G = np.empty(nb), np.empty(nt)
    v = sfh.fg_(True, G, r, H, data, comp)
    # the same diagram as a (100, 200) matrix: Fortran order is the flat layout, C order
    # is converted
    dF = np.asfortranarray(data.reshape(100, 200, order="F"))
    dC = np.ascontiguousarray(dF)
    for d in (dF, dC):
        c2, G2 = np.empty(nb), np.empty(nt)
        assert sfh.fg_(True, G2, r, H, d, c2) == v
        assert np.array_equal(G2, G) and np.array_equal(c2, comp)
    c32 = np.empty(nb, dtype=np.float32)
    G32 = np.empty(nt, dtype=np.float32)
    v32 = sfh.fg_(True, G32, r.astype(np.float32), H, data.astype(np.float32), c32)
    assert np.isfinite(v32) and abs(v32 - v) <= 1e-3 * abs(v)
    c3, G3 = np.empty(nb), np.empty(nt)
    for _ in range(300):
        assert sfh.fg_(True, G3, r, H, data, c3) == v
    assert np.array_equal(G3, G) and np.array_equal(c3, comp)
    assert sfh.fg_(None, G3, r, H, data, c3) is None and np.array_equal(G3, G)


def test_shape_errors_raise_argument_error(sfh):
    M = np.random.default_rng(0).random((10, 3))
    with pytest.raises(ValueError):
        sfh.fg_(True, np.empty(3), np.ones(4), M, np.ones(10), np.empty(10))
    with pytest.raises(ValueError):
        sfh.composite_(np.empty(9), np.ones(3), M)


def test_fit_templates_recovers_noise_free_coefficients(sfh):
    # test/fitting/basic_linear_combinations.jl:47-90 with our own RNG: 10 random
    # 100x100 templates, noise-free data, rtol 1e-7 (LBFGSB) / 1e-6 (BFGS forms).
    rng = np.random.default_rng(58392)
    x = rng.random(10)
    x0 = rng.random(10)
    models = [rng.random((100, 100)) for _ in range(10)]
    data = sum(xi * m for xi, m in zip(x, models))
    M = sfh.stack_models(models)
    H = sfh.Models(M, storage="f64")
    _, xl = sfh.fit_templates_lbfgsb(H, data.ravel(order="F"), x0=x0, factr=1e1, pgtol=1e-12)
    np.testing.assert_allclose(xl, x, rtol=1e-6)
    xf, _ = sfh.fit_templates_fast(H, data.ravel(order="F"), x0=x0, g_abstol=1e-10)
    np.testing.assert_allclose(xf, x, rtol=1e-6)
    res = sfh.fit_templates(H, data.ravel(order="F"), x0=x0, gtol=1e-9)
    np.testing.assert_allclose(res.mle.mu, x, rtol=1e-5)
    # single template, exact answer 3 (basic_linear_combinations.jl:16-25)
    m1 = np.array([[0, 0, 0], [0, 0, 0], [1, 1, 1]], float)
    d1 = np.array([[0, 0, 0], [0, 0, 0], [3, 3, 3]], float)
    _, x1 = sfh.fit_templates_lbfgsb(sfh.stack_models([m1]), d1.ravel(order="F"), x0=[1.0])
    assert x1[0] == pytest.approx(3.0, rel=1e-7)


def test_fit_templates_poisson(sfh):
    # basic_linear_combinations.jl:91-118: x = 100 rand, Poisson data, Julia's vector
    # ≈ with rtol 1e-2 (norm(a - b) <= rtol * max(norm(a), norm(b))).
    rng = np.random.default_rng(1234)
    x = rng.random(10) * 100
    models = [rng.random((100, 100)) for _ in range(10)]
    M = sfh.stack_models(models)
    data = rng.poisson(M @ x).astype(float)
    H = sfh.Models(M, storage="f64")
    _, xl = sfh.fit_templates_lbfgsb(H, data, x0=np.ones(10))
    assert np.linalg.norm(xl - x) <= 1e-2 * np.linalg.norm(x)
    xf, _ = sfh.fit_templates_fast(H, data, x0=np.ones(10))
    assert np.linalg.norm(xf - x) <= 1e-2 * np.linalg.norm(x)
    res = sfh.fit_templates(H, data, x0=np.ones(10))
    assert np.linalg.norm(res.mle.mu - x) <= 1e-2 * np.linalg.norm(x)
    assert np.linalg.norm(res.mle.mu - xf) <= 1e-5 * np.linalg.norm(xf) * 1e2


def test_autotuned_plan_keeps_parity(sfh, O):
    """The autotuner picks a plan among its candidates; fg! with that plan still matches
    the oracle at the FP32-storage tolerances."""
    M, r, data = _problem(60000, 96, seed=7)
    H = sfh.Models(M, storage="f32")
    res = H.autotune(r, data, iters=3)
    ks, R, w2 = res["plan"]
    assert 1 <= ks <= 64 and R in (1024, 2048, 4096) and w2 in (1, 2, 4)
    assert all(t > 0 for t in res["ms"])
    comp = np.empty(M.shape[0])
    G = np.empty(M.shape[1])
    v = sfh.fg_(True, G, r, H, data, comp)
    Mst = M.astype(np.float32).astype(np.float64)
    v_ref, G_ref, w_ref = O.fg(r, Mst, data)
    assert abs(v - v_ref) <= 1e-6 * max(1.0, data.sum() / 1e4)
    scale = np.abs(Mst).T @ np.abs(w_ref) + 1e-300
    assert np.max(np.abs(G - G_ref) / scale) <= 2e-6
