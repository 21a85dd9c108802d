"""Ragged galaxies on the GPU: templates on per-template Hess grids and fg! over a batch of
independent galaxies, against the per-galaxy uniform path and the FP64 oracle.

Tolerances follow the single-vector FP32 tests: composite rtol 2e-6, |ΔlogL| <= 1e-6 per
1e4 stars, gradient error <= 2e-6 of sum_i |M_ij| (|w_i| + n_i/c_i) (the FP32 composite's
relative error enters w = 1 - n/c multiplied by n/c); templates per bin
|gpu - oracle| <= 1e-5 |oracle| + 1e-6 max(oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    if not _t.cuda.is_available():
        pytest.skip("no CUDA device")
    return _t


def _small_ragged(S, ngal=5, seed=3):
    return S.ragged(ngal=ngal, nages=2, nmh=2, nxy=(20, 80), niso=(50, 400), seed=seed)


def test_ragged_templates_match_uniform_batches(sfh, torch):
    """Each galaxy's templates from the ragged call match the uniform batch call on that
    galaxy's own grid (same tiles and star records; the shared-memory atomics of the
    stamps leave the summation order, and so the last bits, to the hardware)."""
    from sfhgpu import synthetic as S
    gals = _small_ragged(S)
    m, mags, offs, lens, dm, edges = S.ragged_isochrones(gals)
    dev = torch.device("cuda", 0)
    d_m, d_mags = torch.as_tensor(m, device=dev), torch.as_tensor(mags, device=dev)
    out, toff = sfh.partial_cmd_smooth_ragged(d_m, d_mags, offs, lens, 1, (0, 1), S.error_models(),
                                              S.completeness_models(), S.imf(), dm, 1.0, edges)
    torch.cuda.synchronize()
    t = 0
    for g in gals:
        nt = g.ntempl
        sl = slice(t, t + nt)
        # the same isochrones, one uniform call per galaxy
        uni = sfh.partial_cmd_smooth_batch(
            d_m, d_mags, offs[sl], lens[sl], 1, (0, 1), S.error_models(),
            S.completeness_models(), S.imf(), dm[sl], 1.0, (g.xedges, g.yedges))
        torch.cuda.synchronize()
        got = out[int(toff[t]):int(toff[t + nt])].view(nt, -1)
        assert got.shape == uni.shape
        tol = 1e-6 * uni.abs() + 1e-7 * uni.abs().amax(dim=1, keepdim=True)
        assert bool(((got - uni).abs() <= tol).all()), f"galaxy starting at template {t}"
        t += nt


def test_ragged_templates_match_oracle(sfh, O, torch):
    from sfhgpu import synthetic as S
    gals = _small_ragged(S, ngal=3, seed=9)
    m, mags, offs, lens, dm, edges = S.ragged_isochrones(gals)
    dev = torch.device("cuda", 0)
    out, toff = sfh.partial_cmd_smooth_ragged(torch.as_tensor(m, device=dev),
                                              torch.as_tensor(mags, device=dev), offs, lens, 1,
                                              (0, 1), S.error_models(), S.completeness_models(),
                                              S.imf(), dm, 1.0, edges)
    out = out.cpu().numpy()
    imf = O.kroupa2001()
    E = [O.ErrModel(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    Cm = [O.ComplModel(c.A, c.m50, c.rho) for c in S.completeness_models()]
    for t in range(lens.size):
        xe, ye = edges[t]
        nx, ny = xe.size - 1, ye.size - 1
        ex = (xe[0], (xe[-1] - xe[0]) / nx, nx)
        ey = (ye[0], (ye[-1] - ye[0]) / ny, ny)
        sl = slice(offs[t], offs[t] + lens[t])
        R = O.partial_cmd_smooth(m[sl], mags[:, sl], E, Cm, 1, (0, 1), imf, dm[t], 1.0,
                                 O.imf_mean(imf), ex, ey)
        G = out[toff[t]:toff[t + 1]].reshape(ny, nx).T
        assert R.sum() > 0
        assert np.all(np.abs(G - R) <= 1e-5 * np.abs(R) + 1e-6 * R.max())


def _ragged_problem(rng, shapes, n_stars=1e4, zero_frac=0.2):
    Ms, rs, ns = [], [], []
    for nb, nt in shapes:
        M = (rng.random((nb, nt)) * (rng.random((nb, nt)) > zero_frac)).astype(np.float32)
        r = np.exp(rng.standard_normal(nt))
        r *= n_stars / (M.astype(np.float64) @ r).sum()
        Ms.append(np.asfortranarray(M))
        rs.append(r)
        ns.append(rng.poisson(M.astype(np.float64) @ r).astype(float))
    return Ms, rs, ns


@pytest.mark.parametrize("seed", [0, 1])
def test_fg_ragged_matches_oracle(sfh, O, torch, seed):
    rng = np.random.default_rng(seed)
    shapes = [(int(rng.integers(50, 300)) * int(rng.integers(50, 300)), int(rng.integers(1, 40)))
              for _ in range(7)] + [(1, 3), (257, 1), (2500, 8), (1024, 16), (1025, 12),
                                    (4096, 32), (1023, 17), (3073, 9)]
    Ms, rs, ns = _ragged_problem(rng, shapes)
    dev = torch.device("cuda", 0)
    packed = torch.as_tensor(np.concatenate([M.ravel(order="F") for M in Ms]), device=dev)
    gal = sfh.Galaxies(packed, [s[0] for s in shapes], [s[1] for s in shapes])
    negL, G, comp = sfh.fg_ragged(gal, np.concatenate(rs), np.concatenate(ns))
    negL, G, comp = negL.cpu().numpy(), G.cpu().numpy(), comp.cpu().numpy()
    # composite alone (G not requested): the model is kept
    _, _, comp_m = sfh.fg_ragged(gal, np.concatenate(rs), np.concatenate(ns), want_grad=False)
    comp_m = comp_m.cpu().numpy()
    for g, (M, r, n) in enumerate(zip(Ms, rs, ns)):
        Mst = M.astype(np.float64)
        v_ref, G_ref, w_ref = O.fg(r, Mst, n)
        b0, b1 = gal.bin_offsets[g], gal.bin_offsets[g + 1]
        t0, t1 = gal.templ_offsets[g], gal.templ_offsets[g + 1]
        np.testing.assert_allclose(comp_m[b0:b1], O.composite(Mst, r), rtol=2e-6, atol=1e-300)
        np.testing.assert_allclose(comp[b0:b1], w_ref, rtol=2e-6, atol=2e-6)
        nst = n.sum()
        assert abs(negL[g] - v_ref) <= 1e-6 * max(1.0, nst / 1e4), (g, negL[g], v_ref)
        scale = np.abs(Mst).T @ (np.abs(w_ref) + np.abs(1.0 - w_ref)) + 1e-300
        assert np.max(np.abs(G[t0:t1] - G_ref) / scale) <= 2e-6


def test_fg_ragged_is_deterministic_and_matches_single_galaxy_path(sfh, torch):
    rng = np.random.default_rng(5)
    shapes = [(60000, 24), (7500, 50)]
    Ms, rs, ns = _ragged_problem(rng, shapes)
    dev = torch.device("cuda", 0)
    packed = torch.as_tensor(np.concatenate([M.ravel(order="F") for M in Ms]), device=dev)
    gal = sfh.Galaxies(packed, [s[0] for s in shapes], [s[1] for s in shapes])
    r, n = np.concatenate(rs), np.concatenate(ns)
    a = [t.cpu().numpy() for t in sfh.fg_ragged(gal, r, n)]
    b = [t.cpu().numpy() for t in sfh.fg_ragged(gal, r, n)]
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    for g, (M, rr, nn) in enumerate(zip(Ms, rs, ns)):
        H = sfh.Models(M, storage="f32")
        Gs = np.empty(M.shape[1])
        v = sfh.fg_(True, Gs, rr, H, nn, np.empty(M.shape[0]))
        assert abs(a[0][g] - v) <= 2e-5 * max(1.0, nn.sum() / 1e4)
        t0, t1 = gal.templ_offsets[g], gal.templ_offsets[g + 1]
        b0, b1 = gal.bin_offsets[g], gal.bin_offsets[g + 1]
        scale = np.abs(M.astype(np.float64)).T @ np.abs(a[2][b0:b1]) + 1e-300
        assert np.max(np.abs(a[1][t0:t1] - Gs) / scale) <= 4e-6


def test_galaxies_reject_bad_descriptors(sfh, torch):
    dev = torch.device("cuda", 0)
    packed = torch.zeros(100, dtype=torch.float32, device=dev)
    with pytest.raises(sfh.SFHArgumentError):
        sfh.Galaxies(packed, [60], [2])          # 120 floats > 100
    with pytest.raises(sfh.SFHArgumentError):
        sfh.Galaxies(packed, [0], [2])           # empty galaxy
    gal = sfh.Galaxies(packed, [50, 25], [1, 2])
    with pytest.raises(ValueError):
        sfh.fg_ragged(gal, np.ones(2), np.ones(75))  # 3 coefficients expected
