"""The allocation-free fg! entry point (sfh_fg_dev_noalloc) against sfh_fg_dev.

Callers that cannot allocate device memory (inside graph-capture regions that must
not allocate, inside host applications that own the device memory budget) use the
variant whose scratch is a fixed array in the library.  This file is collected last
on purpose: it must pass both alone in a fresh process and after every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = float(np.finfo(np.float64).eps)


def _problem(nbins, nt, seed):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > 0.2)
    r = np.exp(rng.standard_normal(nt))
    r *= 1e5 / (M @ r).sum()
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M.astype(np.float32)), r, data


def _reference(sfh, H, d_r, d_n, nbins, nt):
    import torch
    L = sfh.load()
    dev = d_r.device
    c0 = torch.empty(nbins, dtype=torch.float64, device=dev)
    g0 = torch.empty(nt, dtype=torch.float64, device=dev)
    l0 = torch.empty(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    assert L.sfh_fg_dev(H.ctx.handle, H.handle, d_r.data_ptr(), d_n.data_ptr(), c0.data_ptr(),
                        g0.data_ptr(), l0.data_ptr(), EPS) == 0
    H.ctx.synchronize()
    return c0, g0, l0


def _check_twice(sfh, m_ptr, nbins, nt, d_r, d_n, ref, data, scale, want_g=True, want_l=True):
    """Two calls in a row: they share (and must re-arm) the fixed scratch."""
    import torch
    L = sfh.load()
    dev = d_r.device
    c0, g0, l0 = ref
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        c1 = torch.full((nbins,), np.nan, dtype=torch.float64, device=dev)
        g1 = torch.full((nt,), np.nan, dtype=torch.float64, device=dev)
        l1 = torch.full((1,), np.nan, dtype=torch.float64, device=dev)
        rc = L.sfh_fg_dev_noalloc(stream, m_ptr, nbins, nt, d_r.data_ptr(), d_n.data_ptr(),
                                  c1.data_ptr(), g1.data_ptr() if want_g else None,
                                  l1.data_ptr() if want_l else None, EPS)
        assert rc == 0
        torch.cuda.synchronize()
        if want_l:
            # FP32-storage tolerance on logL: 1e-6 per 1e4 stars
            assert abs(l1.item() - l0.item()) <= 1e-6 * max(1.0, data.sum() / 1e4)
        else:
            assert np.isnan(l1.item())  # untouched
        if want_g:
            # composite overwritten with w = 1 - n/c, as fg! does when G is requested
            np.testing.assert_allclose(c1.cpu().numpy(), c0.cpu().numpy(), rtol=2e-6, atol=2e-6)
            assert np.max(np.abs(g1.cpu().numpy() - g0.cpu().numpy()) / (scale + 1e-300)) <= 2e-6
        else:
            assert np.isnan(g1.cpu().numpy()).all()
            # composite holds m = M r when no gradient is requested
            m = c1.cpu().numpy()
            w = 1.0 - data / np.maximum(m, EPS)
            np.testing.assert_allclose(w, c0.cpu().numpy(), rtol=2e-6, atol=2e-6)


@pytest.mark.parametrize("nbins,nt", [(60000, 300), (7501, 37)])
@pytest.mark.parametrize("want_g,want_l", [(True, True), (True, False), (False, True)])
def test_noalloc_matches_fg_dev_twice(sfh, nbins, nt, want_g, want_l):
    import torch
    M32, r, data = _problem(nbins, nt, seed=nbins + nt)
    H = sfh.Models(M32, storage="f32")
    dev = torch.device("cuda", 0)
    d_M = torch.tensor(M32.T.copy(), device=dev)  # (nt, nbins) row-major == column-major M
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    ref = _reference(sfh, H, d_r, d_n, nbins, nt)
    scale = np.abs(M32.astype(np.float64)).T @ np.abs(ref[0].cpu().numpy())
    _check_twice(sfh, d_M.data_ptr(), nbins, nt, d_r, d_n, ref, data, scale, want_g, want_l)


def test_noalloc_offset_pointer(sfh):
    """Templates at a float-aligned but not 16-byte-aligned address (an offset view),
    with nbins a multiple of 4: the call must not use 16-byte vector loads there."""
    import torch
    nbins, nt = 20000, 96
    M32, r, data = _problem(nbins, nt, seed=11)
    H = sfh.Models(M32, storage="f32")
    dev = torch.device("cuda", 0)
    buf = torch.zeros(nbins * nt + 4, dtype=torch.float32, device=dev)
    buf[1:1 + nbins * nt] = torch.tensor(M32.ravel(order="F"), device=dev)
    ptr = buf.data_ptr() + 4
    assert ptr % 16 != 0
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    ref = _reference(sfh, H, d_r, d_n, nbins, nt)
    scale = np.abs(M32.astype(np.float64)).T @ np.abs(ref[0].cpu().numpy())
    _check_twice(sfh, ptr, nbins, nt, d_r, d_n, ref, data, scale)


def test_noalloc_at_the_documented_limits(sfh):
    """nbins = 131072 and ntempl = 4096, the largest shape the fixed scratch admits."""
    import torch
    nbins, nt = 131072, 4096
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    d_M = torch.rand((nt, nbins), generator=g, device=dev, dtype=torch.float32)
    d_M *= (torch.rand((nt, nbins), generator=g, device=dev) > 0.2)
    r = np.exp(np.random.default_rng(5).standard_normal(nt))
    d_r = torch.tensor(r, device=dev)
    m = (d_M.double().T @ d_r)
    d_r *= 1e6 / float(m.sum())
    d_n = torch.poisson((d_M.double().T @ d_r), generator=g)
    data = d_n.cpu().numpy()
    H = sfh.Models.from_device(d_M.data_ptr(), nbins, nt, storage="f32")
    ref = _reference(sfh, H, d_r, d_n, nbins, nt)
    scale = (d_M.double().abs() @ ref[0].abs()).cpu().numpy()
    _check_twice(sfh, d_M.data_ptr(), nbins, nt, d_r, d_n, ref, data, scale)
    H.free()


def test_noalloc_rejects_oversize_without_launching(sfh):
    import torch
    L = sfh.load()
    dev = torch.device("cuda", 0)
    t = torch.zeros(8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    # sizes beyond the fixed scratch: SFH_ERR_SHAPE, checked before any pointer is used
    assert L.sfh_fg_dev_noalloc(stream, t.data_ptr(), 131073, 4, t.data_ptr(), t.data_ptr(),
                                t.data_ptr(), t.data_ptr(), t.data_ptr(), 2.2e-16) == 2
    assert L.sfh_fg_dev_noalloc(stream, t.data_ptr(), 1000, 4097, t.data_ptr(), t.data_ptr(),
                                t.data_ptr(), t.data_ptr(), t.data_ptr(), 2.2e-16) == 2
