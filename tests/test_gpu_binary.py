"""GPU binary-star templates (RandomBinaryPairs) against the FP64 oracle:
binary_hess for a batch of templates (src/StarFormationHistories.jl:627-706) and
partial_cmd_smooth with a binary fraction (:829-910).

Inputs in general position: the synthetic isochrones have round-decimal magnitudes, and a
binary whose companion is negligibly faint has its primary's magnitude to the last bits,
so such a pair can sit on a bin edge to within ulps of log10 / exp10, where two correct FP64
implementations round to opposite sides.  A fixed 1e-6-magnitude jitter of the test
isochrones keeps pairs off the edges.  (The smoothed points themselves sit at bin centres,
which are rounding ties of the stamp's pixel; the oracle and the device form the centre
with the same correctly rounded operations, so they agree there.)

Tolerance: per bin 1e-4 relative + 1e-5 of the template's maximum (FP32 stamps and FP32
completeness / IMF / error evaluations on the GPU against FP64), totals to 1e-5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(gpu, ref, rtol=1e-4, floor=1e-5):
    err = np.abs(gpu - ref)
    bound = rtol * np.abs(ref) + floor * np.abs(ref).max()
    worst = np.max(err / np.maximum(bound, 1e-300))
    assert worst <= 1.0, f"worst normalised error {worst:.3g}"
    assert gpu.sum() == pytest.approx(ref.sum(), rel=1e-5)


def _setup(O):
    from sfhgpu import synthetic as S
    E = [O.ErrModel(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    Cm = [O.ComplModel(c.A, c.m50, c.rho) for c in S.completeness_models()]
    return S, E, Cm


def _isochrones(S, w):
    m_ini, mags, offs, lens = S.isochrone_batch(w)
    mags = mags + 1e-6 * np.random.default_rng(11).random(mags.shape)  # general position
    return m_ini, np.ascontiguousarray(mags), offs, lens


@pytest.mark.parametrize("y_index", [1, 0])
def test_binary_hess_batch_matches_oracle(sfh, O, y_index):
    import torch
    S, E, Cm = _setup(O)
    w = S.small(nages=2, nmh=2)
    m_ini, mags, offs, lens = _isochrones(S, w)
    nx, ny = w.grid
    pts = [sfh.binary_points(m_ini[o:o + n], list(mags[:, o:o + n]), y_index, (0, 1), w.dmod,
                             (w.xedges, w.yedges)) for o, n in zip(offs, lens)]
    md = np.concatenate([p[0] for p in pts])
    gd = np.concatenate([p[1] for p in pts], axis=1)
    ln = np.array([p[0].size for p in pts], dtype=np.int32)
    of = np.concatenate([[0], np.cumsum(ln)[:-1]]).astype(np.int64)
    dev = torch.device("cuda", 0)
    imf = S.imf()
    out = sfh.binary_hess_batch(torch.tensor(md, device=dev), torch.tensor(gd, device=dev), of, ln,
                                y_index, (0, 1), S.error_models(), S.completeness_models(), imf,
                                w.normalize_value, (w.xedges, w.yedges))
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    Oimf = O.kroupa2001()
    ex = (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx)
    ey = (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny)
    for t, (m_ds, g_ds, _) in enumerate(pts):
        R = O.binary_hess(m_ds, g_ds, E, Cm, y_index, (0, 1), Oimf, w.normalize_value,
                          O.imf_mean(Oimf), ex, ey)
        assert R.sum() > 0
        _close(out[t].reshape(ny, nx).T, R)


def test_partial_cmd_smooth_with_binaries_matches_oracle(sfh, O):
    import torch
    S, E, Cm = _setup(O)
    w = S.small(nages=2, nmh=2)
    m_ini, mags, offs, lens = _isochrones(S, w)
    nx, ny = w.grid
    dev = torch.device("cuda", 0)
    out = sfh.partial_cmd_smooth_binary_batch(
        torch.tensor(m_ini, device=dev), torch.tensor(mags, device=dev), offs, lens, 1, (0, 1),
        S.error_models(), S.completeness_models(), S.imf(), w.dmod, w.normalize_value,
        (w.xedges, w.yedges), sfh.RandomBinaryPairs(0.3))
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    Oimf = O.kroupa2001()
    ex = (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx)
    ey = (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny)
    for t in range(w.ntempl):
        sl = slice(offs[t], offs[t] + lens[t])
        R = O.partial_cmd_smooth_binary(m_ini[sl], mags[:, sl], E, Cm, 1, (0, 1), Oimf, w.dmod,
                                        w.normalize_value, O.imf_mean(Oimf), 0.3, ex, ey)
        _close(out[t].reshape(ny, nx).T, R)


def test_binary_hess_needs_y_in_colors(sfh):
    import torch
    from sfhgpu import synthetic as S
    w = S.small()
    dev = torch.device("cuda", 0)
    m = torch.linspace(0.1, 1.0, 20, dtype=torch.float64, device=dev)
    g = torch.ones((3, 20), dtype=torch.float64, device=dev)
    with pytest.raises(Exception):
        sfh.binary_hess_batch(m, g, [0], [20], 2, (0, 1), S.error_models(),
                              S.completeness_models(), S.imf(), 1.0, (w.xedges, w.yedges))
