"""The allocation-free fg! entry point (sfh_fg_dev_noalloc) against sfh_fg_dev.

Callers that cannot allocate device memory (inside graph-capture regions that must
not allocate, inside host applications that own the device memory budget) use the
variant whose scratch is a fixed array in the library.  This file is collected last
on purpose: it must pass both alone in a fresh process and after every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(nbins, nt, seed):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > 0.2)
    r = np.exp(rng.standard_normal(nt))
    r *= 1e5 / (M @ r).sum()
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M.astype(np.float32)), r, data


@pytest.mark.parametrize("nbins,nt", [(60000, 300), (7501, 37)])
def test_noalloc_matches_fg_dev_twice(sfh, nbins, nt):
    import torch
    L = sfh.load()
    M32, r, data = _problem(nbins, nt, seed=nbins + nt)
    H = sfh.Models(M32, storage="f32")
    ctx = H.ctx
    dev = torch.device("cuda", 0)
    d_M = torch.tensor(M32.T.copy(), device=dev)  # (nt, nbins) row-major == column-major M
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    eps = float(np.finfo(np.float64).eps)

    def outs():
        return (torch.empty(nbins, dtype=torch.float64, device=dev),
                torch.empty(nt, dtype=torch.float64, device=dev),
                torch.empty(1, dtype=torch.float64, device=dev))

    c0, g0, l0 = outs()
    torch.cuda.synchronize()
    assert L.sfh_fg_dev(ctx.handle, H.handle, d_r.data_ptr(), d_n.data_ptr(), c0.data_ptr(),
                        g0.data_ptr(), l0.data_ptr(), eps) == 0
    ctx.synchronize()
    stream = torch.cuda.current_stream(dev).cuda_stream
    scale = np.abs(M32.astype(np.float64)).T @ np.abs(c0.cpu().numpy())
    for _ in range(2):  # two calls in a row share (and must re-arm) the fixed scratch
        c1, g1, l1 = outs()
        rc = L.sfh_fg_dev_noalloc(stream, d_M.data_ptr(), nbins, nt, d_r.data_ptr(),
                                  d_n.data_ptr(), c1.data_ptr(), g1.data_ptr(), l1.data_ptr(), eps)
        assert rc == 0
        torch.cuda.synchronize()
        # same tolerances as the FP32-storage parity tests
        assert abs(l1.item() - l0.item()) <= 1e-5 * max(1.0, data.sum() / 1e4)
        np.testing.assert_allclose(c1.cpu().numpy(), c0.cpu().numpy(), rtol=2e-6, atol=2e-6)
        assert np.max(np.abs(g1.cpu().numpy() - g0.cpu().numpy()) / (scale + 1e-300)) <= 2e-6


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
