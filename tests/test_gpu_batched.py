"""GPU parity of the batched tensor-core objective (sfh_fg_batched_dev) against the FP64
oracle evaluated on the same stored values: templates and coefficients as their BF16
hi + lo pairs.

Tolerances reflect FP32 accumulation in tensor memory: the composite carries a relative
error of a few 1e-6 (measured ~4e-6 for 1,200 templates), which enters logL as
~eps * (sum(m) - N); the tests bound |ΔlogL| by 1e-2 per 1e4 stars (+ 1e-7 * |sum m - N|)
and the gradient error by 1e-4 of sum_i |M_ij| |w_i| (W stored as BF16 hi + lo)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_hilo(x):
    """x -> hi + lo with hi = bf16(x), lo = bf16(x - hi) (round to nearest even)."""
    import torch
    t = torch.tensor(np.asarray(x, dtype=np.float32))
    hi = t.to(torch.bfloat16).to(torch.float32)
    lo = (t - hi).to(torch.bfloat16).to(torch.float32)
    return (hi.double() + lo.double()).numpy()


def _bf16_hilo_f64(x):
    import torch
    t = torch.tensor(np.asarray(x, dtype=np.float64))
    hi = t.float().to(torch.bfloat16).double()
    lo = (t - hi).float().to(torch.bfloat16).double()
    return (hi + lo).numpy()


def _problem(nbins, nt, B, seed, n_stars):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > 0.3)
    r0 = np.exp(rng.standard_normal(nt))
    r0 *= n_stars / (M @ r0).sum()
    data = rng.poisson(M @ r0).astype(float)
    R = r0[None, :] * np.exp(0.3 * rng.standard_normal((B, nt)))
    return np.asfortranarray(M.astype(np.float32)), R, data


def _run(sfh, M32, R, data, want_l=True, want_g=True):
    import torch
    L = sfh.load()
    H = sfh.Models(M32, storage="bf16x2")
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
                              d_G.data_ptr() if want_g else None, 2.220446049250313e-16)
    sfh._lib.check(rc, ctx.handle, "sfh_fg_batched_dev")
    ctx.synchronize()
    return (d_L.cpu().numpy() if want_l else None), (d_G.cpu().numpy() if want_g else None)


@pytest.mark.parametrize("nbins,nt,B", [(7500, 50, 128), (20000, 300, 300), (4099, 77, 5),
                                        (60000, 64, 256)])
def test_batched_against_oracle(sfh, O, nbins, nt, B):
    M32, R, data = _problem(nbins, nt, B, seed=nbins + nt + B, n_stars=1e5)
    negL, G = _run(sfh, M32, R, data)
    Ms = np.asfortranarray(_bf16_hilo(M32))
    Rs = _bf16_hilo_f64(R)
    check = np.linspace(0, B - 1, min(B, 6)).astype(int)
    ref_L, ref_G = O.fg_batched(Rs[check], Ms, data, nthreads=4)
    nst = data.sum()
    dL = np.abs(negL[check] - ref_L)
    mism = np.array([abs((Ms @ Rs[b]).sum() - nst) for b in check])
    assert np.all(dL <= 1e-2 * max(1.0, nst / 1e4) + 1e-7 * mism), (dL, nst, mism)
    for k, b in enumerate(check):
        w = 1.0 - data / np.maximum(Ms @ Rs[b], 2.220446049250313e-16)
        scale = np.abs(Ms).T @ np.abs(w) + 1e-300
        assert np.max(np.abs(G[b] - ref_G[k]) / scale) <= 1e-4


def test_batched_logl_only_and_grad_only(sfh, O):
    M32, R, data = _problem(5000, 40, 64, seed=3, n_stars=1e4)
    negL, _ = _run(sfh, M32, R, data, want_l=True, want_g=False)
    _, G = _run(sfh, M32, R, data, want_l=False, want_g=True)
    negL2, G2 = _run(sfh, M32, R, data)
    np.testing.assert_array_equal(negL, negL2)   # deterministic: fixed reduction order
    np.testing.assert_array_equal(G, G2)


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
