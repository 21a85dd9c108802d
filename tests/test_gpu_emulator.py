"""GPU parity of the learned template emulator: the GEMM, the MLP forward / backward
against the FP64 oracle (BF16 operand rounding emulated there), Adam, training, the
transform / reconstruction kernels, the Poisson-deviance score, routing with exact
fallback, and what the trained network gains over the method without it."""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (3, 32, 24, 8)


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    if not _t.cuda.is_available():
        pytest.skip("no CUDA device")
    return _t


@pytest.fixture(scope="module")
def L(sfh):
    return sfh.load()


@pytest.fixture(scope="module")
def ctx(sfh):
    return sfh.default_context()


def _dev(torch, a, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=dtype or np.float32), device="cuda:0")


def _sync(L, ctx):
    assert L.sfh_ctx_synchronize(ctx.handle) == 0


@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("bf16", [0, 1])
def test_gemm_f32_matches_numpy(torch, L, ctx, ta, tb, bf16):
    from test_emulator_host import _bf16
    rng = np.random.default_rng(10 + 2 * ta + tb)
    M, N, K = 70, 131, 45
    A = rng.standard_normal((K, M) if ta else (M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if tb else (K, N)).astype(np.float32)
    C0 = rng.standard_normal((M, N)).astype(np.float32)
    opA = (A.T if ta else A).astype(np.float64)
    opB = (B.T if tb else B).astype(np.float64)
    if bf16:
        opA, opB = _bf16(opA), _bf16(opB)
    ref = 0.5 * opA @ opB + C0
    dA, dB, dC = _dev(torch, A), _dev(torch, B), _dev(torch, C0)
    torch.cuda.synchronize()
    assert L.sfh_gemm_f32(ctx.handle, dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), M, N, K, ta,
                          tb, 1, 0.5, bf16) == 0
    _sync(L, ctx)
    got = dC.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-5 * (np.abs(opA) @ np.abs(opB)).max() + 1e-6


def _net(O, seed, B):
    rng = np.random.default_rng(seed)
    P = (rng.standard_normal(O.mlp_param_count(SHAPE)) * 0.3).astype(np.float32)
    X = rng.uniform(-1, 1, (B, 3)).astype(np.float32)
    T = rng.standard_normal((B, SHAPE[3])).astype(np.float32)
    return P, X, T


@pytest.mark.parametrize("B", [1, 37, 256])
def test_mlp_forward_matches_oracle(torch, L, ctx, O, B):
    P, X, _ = _net(O, 1 + B, B)
    ref = O.mlp_forward(SHAPE, P, X, bf16=True)
    Y = torch.empty((B, SHAPE[3]), dtype=torch.float32, device="cuda:0")
    dP, dX = _dev(torch, P), _dev(torch, X)
    torch.cuda.synchronize()
    assert L.sfh_mlp_forward(ctx.handle, *SHAPE, dP.data_ptr(), dX.data_ptr(), B,
                             Y.data_ptr()) == 0
    got = Y.cpu().numpy()
    # FP32 accumulation and GELU against FP64; a rare BF16 rounding-boundary flip of an
    # activation moves one operand by 2^-8 relative
    assert np.abs(got - ref).max() <= 2e-3 * np.abs(ref).max()
    assert np.median(np.abs(got - ref)) <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("B", [5, 200])
def test_mlp_gradient_matches_oracle(torch, L, ctx, O, B):
    P, X, T = _net(O, 7 + B, B)
    loss_ref, g_ref = O.mlp_loss_grad(SHAPE, P, X, T, bf16=True)
    g = torch.empty(P.size, dtype=torch.float32, device="cuda:0")
    loss = torch.empty(1, dtype=torch.float32, device="cuda:0")
    dP, dX, dT = _dev(torch, P), _dev(torch, X), _dev(torch, T)
    torch.cuda.synchronize()
    assert L.sfh_mlp_loss_grad(ctx.handle, *SHAPE, dP.data_ptr(), dX.data_ptr(), dT.data_ptr(),
                               B, g.data_ptr(), loss.data_ptr()) == 0
    _sync(L, ctx)
    assert loss.item() == pytest.approx(loss_ref, rel=1e-4)
    gg = g.cpu().numpy()
    scale = np.abs(g_ref).max()
    assert np.abs(gg - g_ref).max() <= 3e-3 * scale
    assert np.linalg.norm(gg - g_ref) <= 2e-3 * np.linalg.norm(g_ref)


def test_adam_steps_match_numpy(torch, L, ctx, O):
    """With one training sample every minibatch row is that sample, so the device
    update is reproducible on the host: oracle gradient + bias-corrected Adam."""
    P, X, T = _net(O, 3, 1)
    lr, b1, b2, eps = 3e-3, 0.9, 0.999, 1e-8
    p = P.astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    g1 = None
    for step in range(1, 4):
        _, g = O.mlp_loss_grad(SHAPE, p.astype(np.float32), X, T, bf16=True)
        g1 = g if g1 is None else g1
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    dP, dX, dT = _dev(torch, P), _dev(torch, X), _dev(torch, T)
    dm, dv = torch.zeros_like(dP), torch.zeros_like(dP)
    trace = torch.empty(3, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    assert L.sfh_mlp_train(ctx.handle, *SHAPE, dP.data_ptr(), dm.data_ptr(), dv.data_ptr(), 0,
                           dX.data_ptr(), dT.data_ptr(), 1, 16, 3, lr, 99, trace.data_ptr()) == 0
    got = dP.cpu().numpy()
    # Adam normalises each coordinate, so steps are ~lr regardless of |g|; where a
    # gradient component is ~0 its FP32 sign is noise and the step may go either way
    live = np.abs(g1) > 1e-4 * np.abs(g1).max()
    assert np.abs(got - p)[live].max() <= 0.05 * lr
    assert np.abs(got - p).max() <= 6.5 * lr
    assert np.all(np.diff(trace.cpu().numpy()) < 0)


def test_training_fits_a_smooth_map(torch, L, ctx, O):
    rng = np.random.default_rng(5)
    n = 4096
    X = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    W = rng.standard_normal((3, SHAPE[3]))
    T = np.sin(X @ W).astype(np.float32)
    P, _, _ = _net(O, 11, 1)
    dP, dX, dT = _dev(torch, P * 0.5), _dev(torch, X), _dev(torch, T)
    dm, dv = torch.zeros_like(dP), torch.zeros_like(dP)
    steps = 1500
    trace = torch.empty(steps, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    assert L.sfh_mlp_train(ctx.handle, *SHAPE, dP.data_ptr(), dm.data_ptr(), dv.data_ptr(), 0,
                           dX.data_ptr(), dT.data_ptr(), n, 256, steps, 3e-3, 7,
                           trace.data_ptr()) == 0
    tr = trace.cpu().numpy()
    assert np.all(np.isfinite(tr))
    assert tr[-50:].mean() < 0.1 * tr[:10].mean()
    # the trained net generalises: the oracle forward of the trained weights on fresh points
    Xt = rng.uniform(-1, 1, (512, 3))
    Yt = O.mlp_forward(SHAPE, dP.cpu().numpy(), Xt, bf16=True)
    assert np.mean((Yt - np.sin(Xt @ W)) ** 2) < 0.1 * np.mean(np.sin(Xt @ W) ** 2)


def test_prepare_and_reconstruct_match_numpy(torch, L, ctx):
    rng = np.random.default_rng(2)
    rows, cols, K = 50, 333, 6
    Tm = (rng.gamma(0.3, 1.0, (rows, cols)) * (rng.random((rows, cols)) < 0.6)).astype(np.float32)
    Y = _dev(torch, Tm)
    mean = torch.empty(cols, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    assert L.sfh_emu_prepare(ctx.handle, Y.data_ptr(), rows, cols, 1, mean.data_ptr()) == 0
    _sync(L, ctx)
    s = np.sqrt(Tm.astype(np.float64))
    assert np.allclose(mean.cpu().numpy(), s.mean(0), rtol=1e-6, atol=1e-7)
    assert np.allclose(Y.cpu().numpy(), s - s.mean(0), rtol=1e-5, atol=1e-6)
    coef = rng.standard_normal((rows, K)).astype(np.float32)
    basis = rng.standard_normal((K, cols)).astype(np.float32) * 0.1
    off = rng.standard_normal(cols).astype(np.float32) * 0.3
    out = torch.empty((rows, cols), dtype=torch.float32, device="cuda:0")
    dc, db, do = _dev(torch, coef), _dev(torch, basis), _dev(torch, off)
    torch.cuda.synchronize()
    for mode in (0, 1):
        assert L.sfh_emu_reconstruct(ctx.handle, dc.data_ptr(), db.data_ptr(), do.data_ptr(), K,
                                     cols, rows, mode, out.data_ptr()) == 0
        _sync(L, ctx)
        y = np.maximum(off + coef.astype(np.float64) @ basis, 0)
        ref = y * y if mode == 1 else y
        assert np.allclose(out.cpu().numpy(), ref, rtol=2e-5, atol=1e-6)


def test_deviance_matches_oracle(torch, L, ctx, O):
    rng = np.random.default_rng(4)
    B, nb = 7, 3001
    ex = (rng.gamma(0.4, 1e-4, (B, nb)) * (rng.random((B, nb)) < 0.5)).astype(np.float32)
    em = (ex * np.exp(0.1 * rng.standard_normal((B, nb))) + 1e-7 * rng.random((B, nb)))
    em = em.astype(np.float32)
    em[0, :10] = 0.0  # empty emulated bins hit the floor
    d = torch.empty(B, dtype=torch.float64, device="cuda:0")
    dex, dem = _dev(torch, ex), _dev(torch, em)
    torch.cuda.synchronize()
    assert L.sfh_poisson_deviance(ctx.handle, dex.data_ptr(), dem.data_ptr(), nb, B,
                                  d.data_ptr()) == 0
    _sync(L, ctx)
    ref = [O.poisson_deviance(ex[b], em[b]) for b in range(B)]
    assert np.allclose(d.cpu().numpy(), ref, rtol=1e-9)


# ---------------------------------------------------------------- end to end (small grid)

@pytest.fixture(scope="module")
def trained(torch, sfh, ctx):
    from sfhgpu import emulator as E
    xe, ye = np.linspace(-0.6, 2.4, 41), np.linspace(19.0, 30.0, 51)
    gen = E.SyntheticGenerator(xe, ye, n_iso=200)
    em = E.TemplateEmulator(gen.nbins, ncomp=64, hidden=(256, 256), tol=1e-2, cells=(4, 4, 4),
                            ctx=ctx)
    rep = em.fit(gen, n_train=8192, n_val=2048, steps=3000, batch=1024, lr=1e-3, seed=3)
    return em, gen, rep


def test_emulator_trains_and_reports(trained):
    em, gen, rep = trained
    assert np.all(np.isfinite(rep.loss_trace))
    assert rep.loss_trace[-30:].mean() < 0.2 * rep.loss_trace[:5].mean()
    # a global 64-component basis cannot follow features that translate with distance
    # modulus and age, so even on this coarse grid the median stays near 0.1-0.3
    assert rep.val_deviance_quantiles["q50"] < 0.5


def test_trained_network_beats_the_method_without_it(trained, torch):
    """Without the network the best parameter-free emulator is the PCA mean template;
    the trained MLP must cut the median deviance per star by at least 5x, and emulated
    templates must be built at least 10x faster than exact ones."""
    em, gen, _ = trained
    rng = np.random.default_rng(77)
    th = em.sample_theta(1024, rng)
    exact = gen(th)
    torch.cuda.synchronize()
    emul = em.predict(th)
    d_net = em.score(exact, emul)
    mean_tpl = em.offset.clamp_min(0) ** 2 if em.mode == 1 else em.offset.clamp_min(0)
    d_mean = em.score(exact, mean_tpl.expand(th.shape[0], -1).contiguous())
    assert np.median(d_net) < 0.2 * np.median(d_mean)
    t0 = time.perf_counter()
    gen(th)
    torch.cuda.synchronize()
    t_exact = time.perf_counter() - t0
    t0 = time.perf_counter()
    em.predict(th)
    torch.cuda.synchronize()
    t_emul = time.perf_counter() - t0
    assert t_exact > 10 * t_emul


def test_routing_falls_back_to_exact_templates(trained, torch):
    em, gen, _ = trained
    rng = np.random.default_rng(8)
    th = em.sample_theta(300, rng)
    out, used = em.templates(th, gen, audit=True)
    exact = gen(th)
    d = em.score(exact, em.predict(th))
    assert np.array_equal(used, d <= em.tol)
    # exact templates are reproducible up to the summation order of the stamps' atomics
    def same(a, b):
        return bool(((a - b).abs() <= 1e-6 * b.abs() + 1e-7 * b.abs().amax()).all())

    bad = np.nonzero(~used)[0]
    if bad.size:
        assert same(out[bad], exact[bad])
    good = np.nonzero(used)[0]
    if good.size:
        assert np.all(em.score(exact[good].contiguous(), out[good].contiguous()) <= em.tol)
    # trust-map routing: untrusted cells get exact templates
    out2, used2 = em.templates(th, gen)
    assert np.array_equal(used2, em.trusted(th))
    nb = np.nonzero(~used2)[0]
    if nb.size:
        assert same(out2[nb], exact[nb])


# ---------------------------------------------------------------- grouped (local-basis) form

def test_mlp_forward_rows_matches_oracle(torch, L, ctx, O):
    rng = np.random.default_rng(21)
    G, B = 3, 40
    n = O.mlp_param_count(SHAPE)
    P = (rng.standard_normal((G, n)) * 0.3).astype(np.float32)
    X = rng.uniform(-1, 1, (B, 3)).astype(np.float32)
    grp = rng.integers(0, G, B).astype(np.int32)
    Y = torch.empty((B, SHAPE[3]), dtype=torch.float32, device="cuda:0")
    dP, dX, dg = _dev(torch, P), _dev(torch, X), _dev(torch, grp, np.int32)
    torch.cuda.synchronize()
    assert L.sfh_mlp_forward_rows(ctx.handle, *SHAPE, dP.data_ptr(), G, dX.data_ptr(),
                                  dg.data_ptr(), B, Y.data_ptr()) == 0
    _sync(L, ctx)
    got = Y.cpu().numpy()
    ref = np.stack([O.mlp_forward(SHAPE, P[grp[b]], X[b:b + 1], bf16=True)[0] for b in range(B)])
    assert np.abs(got - ref).max() <= 2e-3 * np.abs(ref).max()
    assert np.median(np.abs(got - ref)) <= 1e-5 * np.abs(ref).max()
    # one group: the row kernel and the GEMM path agree
    Y1 = torch.empty((B, SHAPE[3]), dtype=torch.float32, device="cuda:0")
    assert L.sfh_mlp_forward_rows(ctx.handle, *SHAPE, dP.data_ptr(), 1, dX.data_ptr(), None, B,
                                  Y1.data_ptr()) == 0
    Y2 = torch.empty_like(Y1)
    assert L.sfh_mlp_forward(ctx.handle, *SHAPE, dP.data_ptr(), dX.data_ptr(), B,
                             Y2.data_ptr()) == 0
    _sync(L, ctx)
    assert torch.allclose(Y1, Y2, rtol=1e-5, atol=1e-6)


def test_grouped_adam_matches_numpy(torch, L, ctx, O):
    """Two groups with one sample each: every minibatch row of a group is its sample, so
    each group's update is the oracle gradient + Adam (the loss is averaged over groups,
    which Adam's per-coordinate normalisation ignores)."""
    rng = np.random.default_rng(22)
    G = 2
    n = O.mlp_param_count(SHAPE)
    P = (rng.standard_normal((G, n)) * 0.3).astype(np.float32)
    X = rng.uniform(-1, 1, (G, 3)).astype(np.float32)
    T = rng.standard_normal((G, SHAPE[3])).astype(np.float32)
    lr = 3e-3
    ref, live = [], []
    for g in range(G):
        p = P[g].astype(np.float64)
        m = np.zeros_like(p)
        v = np.zeros_like(p)
        for step in range(1, 4):
            _, gr = O.mlp_loss_grad(SHAPE, p.astype(np.float32), X[g:g + 1], T[g:g + 1], True)
            if step == 1:
                live.append(np.abs(gr) > 1e-4 * np.abs(gr).max())
            m = 0.9 * m + 0.1 * gr
            v = 0.999 * v + 0.001 * gr * gr
            p = p - lr * (m / (1 - 0.9 ** step)) / (np.sqrt(v / (1 - 0.999 ** step)) + 1e-8)
        ref.append(p)
    dP, dX, dT = _dev(torch, P), _dev(torch, X), _dev(torch, T)
    dm, dv = torch.zeros_like(dP), torch.zeros_like(dP)
    off = np.array([0, 1, 2], dtype=np.int64)
    torch.cuda.synchronize()
    assert L.sfh_mlp_train_grouped(ctx.handle, *SHAPE, G, dP.data_ptr(), dm.data_ptr(),
                                   dv.data_ptr(), 0, dX.data_ptr(), dT.data_ptr(), off.ctypes.data,
                                   8, 3, lr, 5, None) == 0
    got = dP.cpu().numpy()
    for g in range(G):
        # near-zero gradient components: FP32 sign noise, see test_adam_steps_match_numpy
        assert np.abs(got[g] - ref[g])[live[g]].max() <= 0.05 * lr
        assert np.abs(got[g] - ref[g]).max() <= 6.5 * lr
    # every group must own at least one sample
    bad = np.array([0, 1, 1], dtype=np.int64)
    assert L.sfh_mlp_train_grouped(ctx.handle, *SHAPE, G, dP.data_ptr(), dm.data_ptr(),
                                   dv.data_ptr(), 0, dX.data_ptr(), dT.data_ptr(), bad.ctypes.data,
                                   8, 1, lr, 5, None) != 0


def test_reconstruct_rows_matches_numpy(torch, L, ctx):
    rng = np.random.default_rng(23)
    G, K, nb, B = 4, 5, 777, 33
    coef = rng.standard_normal((B, K)).astype(np.float32)
    basis = (rng.standard_normal((G, K, nb)) * 0.1).astype(np.float32)
    off = (rng.standard_normal((G, nb)) * 0.3).astype(np.float32)
    grp = rng.integers(0, G, B).astype(np.int32)
    out = torch.empty((B, nb), dtype=torch.float32, device="cuda:0")
    d = [_dev(torch, a) for a in (coef, basis, off)]
    dg = _dev(torch, grp, np.int32)
    torch.cuda.synchronize()
    for mode in (0, 1):
        assert L.sfh_emu_reconstruct_rows(ctx.handle, d[0].data_ptr(), dg.data_ptr(), G,
                                          d[1].data_ptr(), d[2].data_ptr(), K, nb, B, mode,
                                          out.data_ptr()) == 0
        _sync(L, ctx)
        y = np.maximum(off[grp] + np.einsum("bk,bki->bi", coef.astype(np.float64), basis[grp]), 0)
        ref = y * y if mode == 1 else y
        assert np.allclose(out.cpu().numpy(), ref, rtol=2e-5, atol=1e-6)


@pytest.mark.parametrize("K,nb", [(5, 777), (64, 1024), (130, 2048), (1, 3), (1, 4)])
def test_reconstruct_groups_matches_rows(torch, L, ctx, K, nb):
    """The segment kernel (one basis read per cell segment; float4 rows when nbins % 4 == 0,
    scalar otherwise; 4-, 8- and 16-row accumulators) gives the per-row kernel's bits."""
    from sfhgpu.emulator import group_segments
    rng = np.random.default_rng(K)
    G = 6
    grp = np.concatenate([np.full(n, g) for g, n in enumerate([1, 3, 7, 16, 21, 40])])
    grp = rng.permutation(grp).astype(np.int32)
    B = grp.size
    coef = rng.standard_normal((B, K)).astype(np.float32)
    basis = (rng.standard_normal((G, K, nb)) * 0.1).astype(np.float32)
    off = (rng.standard_normal((G, nb)) * 0.3).astype(np.float32)
    d = [_dev(torch, a) for a in (coef, basis, off)]
    dg = _dev(torch, grp, np.int32)
    rows, seg = group_segments(grp)
    assert seg[:, 2].max() == 16 and seg[:, 2].min() == 1
    dr, ds = _dev(torch, rows, np.int32), _dev(torch, seg, np.int32)
    ref = torch.empty((B, nb), dtype=torch.float32, device="cuda:0")
    out = torch.full((B, nb), -1.0, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    for mode in (0, 1):
        assert L.sfh_emu_reconstruct_rows(ctx.handle, d[0].data_ptr(), dg.data_ptr(), G,
                                          d[1].data_ptr(), d[2].data_ptr(), K, nb, B, mode,
                                          ref.data_ptr()) == 0
        assert L.sfh_emu_reconstruct_groups(ctx.handle, d[0].data_ptr(), dr.data_ptr(),
                                            ds.data_ptr(), seg.shape[0], G, d[1].data_ptr(),
                                            d[2].data_ptr(), K, nb, B, mode,
                                            out.data_ptr()) == 0
        _sync(L, ctx)
        assert torch.equal(out, ref)
    # a segment naming a group out of range writes NaN to its rows and nothing else
    bad = seg.copy()
    bad[0, 0] = G
    ds = _dev(torch, bad, np.int32)
    out.fill_(-1.0)
    torch.cuda.synchronize()
    assert L.sfh_emu_reconstruct_groups(ctx.handle, d[0].data_ptr(), dr.data_ptr(),
                                        ds.data_ptr(), bad.shape[0], G, d[1].data_ptr(),
                                        d[2].data_ptr(), K, nb, B, 1, out.data_ptr()) == 0
    _sync(L, ctx)
    nanrows = rows[bad[0, 1]:bad[0, 1] + bad[0, 2]]
    assert bool(torch.isnan(out[torch.as_tensor(nanrows, device="cuda:0")]).all())
    keep = np.setdiff1d(np.arange(B), nanrows)
    assert torch.equal(out[torch.as_tensor(keep, device="cuda:0")],
                       ref[torch.as_tensor(keep, device="cuda:0")])


@pytest.fixture(scope="module")
def trained_local(torch, sfh, ctx):
    from sfhgpu import emulator as E
    xe, ye = np.linspace(-0.6, 2.4, 41), np.linspace(19.0, 30.0, 51)
    gen = E.SyntheticGenerator(xe, ye, n_iso=200)
    em = E.TemplateEmulator(gen.nbins, ncomp=64, hidden=(256, 256), tol=1e-2,
                            basis_cells=(2, 2, 4), ctx=ctx)
    rep = em.fit(gen, n_train=8192, n_val=2048, steps=3000, lr=1e-3, seed=3, batch_per_cell=64)
    return em, gen, rep


def test_local_bases_beat_the_global_basis(trained, trained_local, torch):
    """Per-cell bases and networks follow features that move with theta better than one
    global basis: lower median deviance per star on the same held-out templates."""
    em_g, gen, _ = trained
    em_l, _, rep = trained_local
    assert np.all(np.isfinite(rep.loss_trace))
    rng = np.random.default_rng(99)
    th = em_g.sample_theta(1024, rng)
    exact = gen(th)
    d_g = em_g.score(exact, em_g.predict(th))
    d_l = em_l.score(exact, em_l.predict(th))
    assert np.median(d_l) < 0.5 * np.median(d_g)
    # and the local networks beat the local mean templates (no network)
    grp = torch.as_tensor(em_l.group_of(th), device=exact.device)
    y = em_l.offset[grp].clamp_min(0)
    d_mean = em_l.score(exact, (y * y).contiguous())
    assert np.median(d_l) < 0.2 * np.median(d_mean)


@pytest.fixture(scope="module")
def trained_fixed(torch, sfh, ctx):
    """An emulator for one distance (modulus 27 +- 0.05), the way a fit of one galaxy uses
    it: per-cell bases over (log age, [M/H]) only."""
    from sfhgpu import emulator as E
    xe, ye = np.linspace(-0.6, 2.4, 41), np.linspace(19.0, 30.0, 51)
    gen = E.SyntheticGenerator(xe, ye, n_iso=200)
    em = E.TemplateEmulator(gen.nbins, ncomp=64, hidden=(256, 256), tol=1e-2,
                            bounds=((6.6, 10.1), (-2.5, 0.3), (26.95, 27.05)),
                            basis_cells=(4, 2, 1), trust_cells=(8, 4, 1), ctx=ctx)
    rep = em.fit(gen, n_train=8192, n_val=2048, steps=3000, lr=1e-3, seed=5, batch_per_cell=64)
    return em, gen, rep


def test_no_requests_give_empty_templates(trained_fixed, torch):
    em, gen, _ = trained_fixed
    none = np.empty((0, 3))
    assert tuple(em.coefficients(none).shape) == (0, em.K)
    assert tuple(em.predict(none).shape) == (0, em.nbins)
    out, used = em.templates(none, gen)
    assert tuple(out.shape) == (0, em.nbins) and used.size == 0


def test_routed_templates_fit_like_exact_templates(trained_fixed, torch, sfh):
    """The gain against the exact-template path at the tolerance: a fit on routed templates
    (emulated where the trust map allows, exact elsewhere) builds fewer exact templates, and
    its optimum, scored on the exact templates, is within tol x stars of the exact-template
    fit's optimum (the Poisson deviance of the composite of templates that each sit within
    tol per star of the exact ones is at most tol per star, by joint convexity)."""
    from sfhgpu.fitting import fit_templates_fast
    em, gen, _ = trained_fixed
    assert em.cells == (8, 4, 1) and em.trust.size == 32   # the trust map's own grid
    rng = np.random.default_rng(41)
    th = em.sample_theta(4096, rng)
    tr = em.trusted(th)
    assert tr.any(), "no trusted cell at tol 1e-2"
    th = np.concatenate([th[tr][:24], th[~tr][:24]])
    B = th.shape[0]
    exact = gen(th)
    routed, used = em.templates(th, gen)
    torch.cuda.synchronize()
    assert used.any() and (~used).sum() < B      # exact templates built: fewer than requested
    X = exact.double().cpu().numpy().T            # (nbins, B)
    Xr = routed.cpu().numpy().T.astype(np.float64)
    c = np.exp(rng.standard_normal(B))
    c *= 1e5 / (X @ c).sum()
    data = rng.poisson(X @ c).astype(np.float64)
    nstars = data.sum()

    def nll(M, x):
        m = np.maximum(M @ x, 1e-300)
        pos = data > 0
        return float(np.sum(m - data) + np.sum(data[pos] * np.log(data[pos] / m[pos])))

    c_x, _ = fit_templates_fast(sfh.Models(np.asfortranarray(X)), data, g_abstol=1e-6)
    c_r, _ = fit_templates_fast(sfh.Models(np.asfortranarray(Xr)), data, g_abstol=1e-6)
    gap = nll(X, c_r) - nll(X, c_x)
    assert -1e-6 * nstars <= gap <= em.tol * nstars
    assert abs(c_r.sum() / c_x.sum() - 1.0) < 0.05


def test_local_routing_falls_back_to_exact_templates(trained_local, torch):
    em, gen, _ = trained_local
    rng = np.random.default_rng(18)
    th = em.sample_theta(200, rng)
    out, used = em.templates(th, gen, audit=True)
    exact = gen(th)
    d = em.score(exact, em.predict(th))
    assert np.array_equal(used, d <= em.tol)
    bad = np.nonzero(~used)[0]
    if bad.size:
        assert bool(((out[bad] - exact[bad]).abs()
                     <= 1e-6 * exact[bad].abs() + 1e-7 * exact[bad].abs().amax()).all())
