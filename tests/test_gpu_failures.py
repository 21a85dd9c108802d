"""Failure detection without a GPU fault.

A bounded device wait made to run out (a bulk copy that is never issued, so nothing
completes the barrier the consumers wait on) returns SFH_ERR_TIMEOUT and the next call on
the same context succeeds; a refused allocation returns SFH_ERR_NOMEM; non-finite
coefficients return SFH_ERR_NUMERIC with NaN results, as the reference's arithmetic would
give.  Every failure here is made on the host or by a wait that gives up."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(nbins=20000, nt=200, seed=5, n_stars=1e5):
    rng = np.random.default_rng(seed)
    M = rng.random((nbins, nt)) * (rng.random((nbins, nt)) > 0.3)
    r = np.exp(rng.standard_normal(nt))
    r *= n_stars / (M @ r).sum()
    data = rng.poisson(M @ r).astype(float)
    return np.asfortranarray(M), r, data


def _fg(sfh, H, r, data):
    comp = np.empty(H.nbins)
    G = np.empty(H.nt)
    v = sfh.fg_(True, G, r, H, data, comp)
    return v, G


def test_wait_that_runs_out_returns_timeout_and_the_context_recovers(sfh, O):
    from sfhgpu._lib import SFH_ERR_TIMEOUT, SFH_INJECT_DROP_COPY, SFHError
    M, r, data = _problem()
    ctx = sfh.Context(0)
    H = sfh.Models(M, storage="f32", ctx=ctx)
    H.set_path("onepass")
    v0, G0 = _fg(sfh, H, r, data)
    ctx.set_wait_budget(2_000_000)  # about 1 ms
    ctx.inject_fault(SFH_INJECT_DROP_COPY)
    with pytest.raises(SFHError) as e:
        _fg(sfh, H, r, data)
    assert e.value.status == SFH_ERR_TIMEOUT
    # the next call on the same context: correct results, no error left behind
    v1, G1 = _fg(sfh, H, r, data)
    ctx.set_wait_budget(0)
    v2, G2 = _fg(sfh, H, r, data)
    assert v1 == v0 and v2 == v0
    np.testing.assert_array_equal(G1, G0)
    v_ref, _, _ = O.fg(r, M.astype(np.float32).astype(np.float64), data)
    assert abs(v2 - v_ref) <= 1e-6 * data.sum() / 1e4
    ctx.synchronize()


def test_refused_allocation_returns_nomem_and_the_next_call_succeeds(sfh):
    from sfhgpu._lib import SFH_ERR_NOMEM, SFH_INJECT_ALLOC_FAIL, SFHError
    M, r, data = _problem(nbins=5000, nt=40)
    ctx = sfh.Context(0)
    H = sfh.Models(M, storage="f32", ctx=ctx)
    ctx.inject_fault(SFH_INJECT_ALLOC_FAIL)  # the context has no staging yet: fg! allocates
    with pytest.raises(SFHError) as e:
        _fg(sfh, H, r, data)
    assert e.value.status == SFH_ERR_NOMEM
    v, G = _fg(sfh, H, r, data)
    assert np.isfinite(v) and np.all(np.isfinite(G))


def test_non_finite_coefficients_return_numeric(sfh):
    import ctypes as C
    from sfhgpu._lib import SFH_ERR_NUMERIC
    M, r, data = _problem(nbins=5000, nt=40)
    H = sfh.Models(M, storage="f32")
    L = sfh.load()
    for bad in (np.nan, np.inf):
        rb = r.copy()
        rb[7] = bad
        comp = np.empty(H.nbins)
        G = np.zeros(H.nt)
        out = C.c_double(0.0)
        rc = L.sfh_fg(H.ctx.handle, H.handle, 0, rb.ctypes.data, data.ctypes.data,
                      comp.ctypes.data, G.ctypes.data, C.byref(out))
        assert rc == SFH_ERR_NUMERIC
        assert np.isnan(out.value) and np.isnan(G).all()
    v, G = _fg(sfh, H, r, data)  # finite coefficients: fine
    assert np.isfinite(v)
