"""GPU parity for bin_cmd_smooth / addstar! / partial_cmd_smooth against the FP64 oracle.

Tolerance (FP32 templates vs FP64 oracle): per bin |gpu - ref| <= 1e-5 |ref| + 1e-6 max(ref)
(relative 1e-5, with an absolute floor for far-tail bins that FP32 erf cannot resolve)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(gpu, ref, rtol=1e-5, floor=1e-6):
    err = np.abs(gpu - ref)
    bound = rtol * np.abs(ref) + floor * np.abs(ref).max()
    worst = np.max(err / np.maximum(bound, 1e-300))
    assert worst <= 1.0, f"worst normalised error {worst:.3g}"


def _random_stars(rng, n, xr, yr, smin, smax):
    x = rng.uniform(*xr, n)
    y = rng.uniform(*yr, n)
    sx = np.exp(rng.uniform(np.log(smin), np.log(smax), n))
    sy = np.exp(rng.uniform(np.log(smin), np.log(smax), n))
    w = rng.random(n) + 0.1
    return x, y, sx, sy, w


@pytest.mark.parametrize("cov", [0, 1, -1])
@pytest.mark.parametrize("nx,ny", [(75, 100), (200, 300), (33, 17)])
def test_bin_cmd_smooth_random(sfh, O, cov, nx, ny):
    rng = np.random.default_rng(nx * 7 + ny + cov)
    xe = np.linspace(-0.6, 2.4, nx + 1)
    ye = np.linspace(19.0, 30.0, ny + 1)
    # include stars beyond the grid edges so clipping is exercised
    x, y, sx, sy, w = _random_stars(rng, 300, (-0.8, 2.6), (18.5, 30.5), 0.003, 0.4)
    H = sfh.bin_cmd_smooth(x, y, sx, sy, cov, weights=w, edges=(xe, ye)).weights
    R = O.bin_cmd_smooth(x, y, sx, sy, w, cov, (xe[0], (xe[-1] - xe[0]) / nx, nx),
                         (ye[0], (ye[-1] - ye[0]) / ny, ny))
    assert H.shape == (nx, ny)
    _close(H, R)


def test_edge_cases(sfh, O):
    xe = np.linspace(0.0, 1.0, 11)   # step 0.1, 10 bins
    ye = np.linspace(0.0, 2.0, 21)   # step 0.1, 20 bins
    ex = (0.0, 0.1, 10)
    ey = (0.0, 0.1, 20)
    cases = {
        # centroid exactly on a .5 pixel coordinate: ties-to-even rounding of x0 = 3.5, 4.5
        "ties": ([0.25, 0.35], [1.05, 1.05], [0.02, 0.02], [0.02, 0.02]),
        # window clipped to one column at the grid edge: skipped by the reference (:359)
        "one_column": ([1.2], [1.0], [0.001], [0.05]),
        # star far outside: nothing
        "outside": ([5.0], [5.0], [0.01], [0.01]),
        # vanishing sigma: the bin-integrated Gaussian becomes a hard histogram
        "tiny_sigma": ([0.47], [1.13], [1e-9], [1e-9]),
        # huge sigma: window covers the whole grid
        "huge_sigma": ([0.5], [1.0], [3.0], [3.0]),
    }
    for name, (x, y, sx, sy) in cases.items():
        w = np.ones(len(x))
        for cov in (0, 1):
            H = sfh.bin_cmd_smooth(x, y, sx, sy, cov, weights=w, edges=(xe, ye)).weights
            R = O.bin_cmd_smooth(x, y, sx, sy, w, cov, ex, ey)
            _close(H, R)
    # empty star list: all-zero template
    H = sfh.bin_cmd_smooth([], [], [], [], 0, weights=[], edges=(xe, ye)).weights
    assert H.shape == (10, 20) and not H.any()
    with pytest.raises(ValueError):
        sfh.bin_cmd_smooth([0.5], [1.0], [0.1], [0.1], 2, edges=(xe, ye))


def _batch_vs_oracle(sfh, O, w, y_index, color_indices, ntest=None):
    import torch
    from sfhgpu import synthetic as S
    m_ini, mags, offs, lens = S.isochrone_batch(w)
    dev = torch.device("cuda", 0)
    imf = S.imf()
    out = sfh.partial_cmd_smooth_batch(
        torch.tensor(m_ini, device=dev), torch.tensor(mags, device=dev), offs, lens, y_index,
        color_indices, S.error_models(), S.completeness_models(), imf, w.dmod,
        w.normalize_value, (w.xedges, w.yedges))
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    nx, ny = w.grid
    Oimf = O.kroupa2001()
    E = [O.ErrModel(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    Cm = [O.ComplModel(c.A, c.m50, c.rho) for c in S.completeness_models()]
    ex = (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx)
    ey = (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny)
    idx = range(w.ntempl) if ntest is None else np.linspace(0, w.ntempl - 1, ntest).astype(int)
    for t in idx:
        sl = slice(offs[t], offs[t] + lens[t])
        R = O.partial_cmd_smooth(m_ini[sl], mags[:, sl], E, Cm, y_index, color_indices, Oimf,
                                 w.dmod, w.normalize_value, O.imf_mean(Oimf), ex, ey)
        G = out[t].reshape(ny, nx).T
        assert R.sum() > 0
        _close(G, R)


@pytest.mark.parametrize("y_index,ci", [(1, (0, 1)), (0, (0, 1)), (2, (0, 1))])
def test_partial_cmd_smooth_batch_small(sfh, O, y_index, ci):
    from sfhgpu import synthetic as S
    _batch_vs_oracle(sfh, O, S.small(), y_index, ci)


def test_partial_cmd_smooth_batch_config1(sfh, O):
    from sfhgpu import synthetic as S
    _batch_vs_oracle(sfh, O, S.config1(), 1, (0, 1), ntest=6)


def test_partial_cmd_smooth_host_callables(sfh, O):
    """partial_cmd_smooth with Python callables (host preprocessing, GPU stamps)."""
    from sfhgpu import synthetic as S
    w = S.small()
    la, mh = w.template_params
    m, mags = S.isochrone(la[1], mh[1], w.n_iso)
    H = sfh.partial_cmd_smooth(m, list(mags), S.error_funcs(), 2, (0, 1), S.imf(),
                               S.completeness_funcs(), dmod=w.dmod,
                               edges=(w.xedges, w.yedges)).weights
    nx, ny = w.grid
    Oimf = O.kroupa2001()
    R = O.partial_cmd_smooth(m, mags, [O.ErrModel(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()],
                             [O.ComplModel(c.A, c.m50, c.rho) for c in S.completeness_models()],
                             2, (0, 1), Oimf, w.dmod, 1.0, O.imf_mean(Oimf),
                             (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx),
                             (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny))
    _close(H, R)


@pytest.mark.parametrize("y_index,branch", [(1, "covariant"), (2, "separable")])
def test_partial_cmd_smooth_production_grid(sfh, O, y_index, branch):
    """The production workload: all 1,200 templates (40 log-ages x 30 [M/H]) on the 200 x 300
    grid built in FP32 on the GPU, 24 of them spread over the age-metallicity grid checked
    against the FP64 oracle (y = V inside the colour B - V: the covariant kernel; y = R: the
    separable kernel)."""
    import torch
    from sfhgpu import synthetic as S
    w = S.config2()
    m_ini, mags, offs, lens = S.isochrone_batch(w)
    dev = torch.device("cuda", 0)
    out = sfh.partial_cmd_smooth_batch(
        torch.tensor(m_ini, device=dev), torch.tensor(mags, device=dev), offs, lens, y_index,
        (0, 1), S.error_models(), S.completeness_models(), S.imf(), w.dmod, w.normalize_value,
        (w.xedges, w.yedges))
    torch.cuda.synchronize()
    assert out.shape[0] == 1200
    nx, ny = w.grid
    ex = (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx)
    ey = (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny)
    err = [(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    com = [(c.A, c.m50, c.rho) for c in S.completeness_models()]
    # 6 ages x 4 metallicities, corners included
    ia = np.linspace(0, w.logAges.size - 1, 6).astype(int)
    im = np.linspace(0, w.MHs.size - 1, 4).astype(int)
    idx = [a * w.MHs.size + z for a in ia for z in im]
    jobs = [(m_ini[offs[t]:offs[t] + lens[t]], mags[:, offs[t]:offs[t] + lens[t]], err, com,
             y_index, (0, 1), w.dmod, w.normalize_value, ex, ey) for t in idx]
    refs = O.partial_cmd_smooth_many(jobs)
    gpu = out[idx].cpu().numpy()
    for k, t in enumerate(idx):
        R = refs[k]
        assert R.sum() > 0
        _close(gpu[k].reshape(ny, nx).T, R)
