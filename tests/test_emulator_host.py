"""CPU checks of the learned emulator's test infrastructure and host logic: the FP64 MLP
restatement's analytic gradient against central finite differences, its BF16 operand
rounding, the Poisson-deviance score, and the emulator's routing bookkeeping."""
import numpy as np
import pytest

SHAPE = (3, 16, 12, 5)


def _net(O, seed=0, B=9):
    rng = np.random.default_rng(seed)
    P = rng.standard_normal(O.mlp_param_count(SHAPE)) * 0.4
    X = rng.uniform(-1, 1, (B, 3))
    T = rng.standard_normal((B, SHAPE[3]))
    return P, X, T


def test_mlp_param_count(O):
    i, h1, h2, o = SHAPE
    assert O.mlp_param_count(SHAPE) == h1 * i + h1 + h2 * h1 + h2 + o * h2 + o
    assert O.mlp_param_count((3, 256, 256, 64)) == 83_264


def test_oracle_mlp_gradient_matches_finite_differences(O):
    P, X, T = _net(O)
    loss, g = O.mlp_loss_grad(SHAPE, P, X, T, bf16=False)
    Y = O.mlp_forward(SHAPE, P, X, bf16=False)
    assert abs(((Y - T) ** 2).mean() - loss) < 1e-14
    h = 1e-6
    fd = np.empty_like(g)
    for k in range(P.size):
        e = np.zeros_like(P)
        e[k] = h
        fd[k] = (O.mlp_loss_grad(SHAPE, P + e, X, T, False)[0]
                 - O.mlp_loss_grad(SHAPE, P - e, X, T, False)[0]) / (2 * h)
    assert np.abs(fd - g).max() <= 1e-8 * max(1.0, np.abs(g).max())


def _bf16(x):
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def test_oracle_bf16_mode_rounds_operands(O):
    # a single linear layer (GELU-free path): the output layer of a net whose hidden
    # activations are known -- compare the BF16 forward with numpy on rounded operands
    P, X, _ = _net(O, seed=3)
    i, h1, h2, o = SHAPE
    W1 = P[: h1 * i].reshape(h1, i)
    b1 = P[h1 * i: h1 * i + h1]
    from math import erf, sqrt
    gelu = np.vectorize(lambda z: 0.5 * z * (1 + erf(z / sqrt(2))))
    A1 = gelu(_bf16(X) @ _bf16(W1).T + b1)
    off = h1 * i + h1
    W2 = P[off: off + h2 * h1].reshape(h2, h1)
    b2 = P[off + h2 * h1: off + h2 * h1 + h2]
    A2 = gelu(_bf16(A1) @ _bf16(W2).T + b2)
    off += h2 * h1 + h2
    W3 = P[off: off + o * h2].reshape(o, h2)
    b3 = P[off + o * h2:]
    Y = _bf16(A2) @ _bf16(W3).T + b3
    assert np.allclose(O.mlp_forward(SHAPE, P, X, bf16=True), Y, rtol=1e-12, atol=1e-12)
    # and BF16 rounding is ties-to-even on the 16 dropped bits
    assert _bf16(np.float32(1.0) + np.float32(2.0 ** -8)) == 1.0
    assert _bf16(np.float32(1.0) + np.float32(3 * 2.0 ** -8)) == 1.0 + 2.0 ** -6


def test_poisson_deviance_oracle(O):
    rng = np.random.default_rng(1)
    t = rng.gamma(0.5, 1.0, 500) * (rng.random(500) < 0.7)
    e = t * np.exp(0.05 * rng.standard_normal(500)) + 1e-4
    ref = 2 * np.sum(e - t + np.where(t > 0, t * np.log(np.where(t > 0, t, 1) / e), 0)) / t.sum()
    assert O.poisson_deviance(t, e) == pytest.approx(ref, rel=1e-12)
    assert O.poisson_deviance(t, t) < 1e-25  # only the 1e-30 floor of empty bins remains


def test_emulator_trust_map_routing():
    from sfhgpu import emulator as E
    em = E.TemplateEmulator.__new__(E.TemplateEmulator)
    em.bounds = np.asarray(((6.6, 10.1), (-2.5, 0.3), (24.0, 30.0)))
    em.cells = (2, 2, 2)
    em.tol = 1e-3
    th = np.array([[7.0, -2.0, 25.0], [7.1, -2.1, 25.5], [9.0, 0.0, 29.0], [12.0, 0.0, 25.0]])
    em._build_trust(th[:3], np.array([1e-4, 5e-4, 2e-3]))
    # the first two share a cell (worst 5e-4 <= tol); the third fails; outside the box and
    # unvalidated cells are never trusted
    assert list(em.trusted(th)) == [True, True, False, False]
    assert not em.trusted(np.array([[9.5, -2.0, 25.0]]))[0]
    assert np.allclose(em.standardize([[6.6, -2.5, 24.0], [10.1, 0.3, 30.0]]),
                       [[-1, -1, -1], [1, 1, 1]])


@pytest.mark.parametrize("n,ngroups,max_rows", [(1, 1, 16), (37, 3, 16), (500, 11, 16),
                                                 (64, 1, 16), (90, 5, 4)])
def test_group_segments_cover_every_row_once(n, ngroups, max_rows):
    """Row segments for the cell-grouped reconstruction: every row in exactly one segment,
    each segment one group, 1..max_rows rows, rows sorted by group (stable)."""
    from sfhgpu.emulator import group_segments
    g = np.random.default_rng(n).integers(0, ngroups, n)
    rows, seg = group_segments(g, max_rows=max_rows)
    assert rows.dtype == np.int32 and seg.dtype == np.int32 and seg.shape[1] == 3
    assert np.array_equal(rows, np.argsort(g, kind="stable"))
    seen = np.zeros(n, int)
    for grp, start, count in seg:
        assert 1 <= count <= max_rows
        assert np.all(g[rows[start:start + count]] == grp)
        seen[rows[start:start + count]] += 1
    assert np.all(seen == 1)
    # segments are as long as they may be: one short segment per group at most
    for grp in np.unique(g):
        c = seg[seg[:, 0] == grp, 2]
        assert np.sum(c < max_rows) <= 1 and c.sum() == np.sum(g == grp)
