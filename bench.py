#!/usr/bin/env python
"""Benchmark of the Hess-diagram hot path on one GB300 (replicas on N GPUs).

Workload (the production-size configuration): 1,200 templates (40 log-ages 6.6-10.1 x
30 [M/H] -2.5..0.3) built on the GPU by partial_cmd_smooth (V vs B-V, covariant kernel)
on a 200 x 300 Hess grid, stored FP32; one observed diagram holding 1e6 stars.

A step is one fg! evaluation (composite!, loglikelihood, ∇loglikelihood!) of one
coefficient vector against the 60,000 x 1,200 template matrix.  The matrix is 288 MB,
but the occupied-bin plan streams only the occupied bins' rows (66 MB), which fit in L2
(129 MB): L2 is flushed before every timed step, outside the step's CUDA-event interval.

  value : evals/s with inputs resident in HBM (sfh_fg_dev): the sum of the steps' CUDA-event
          intervals on the context stream
  e2e   : evals/s through the public host-array call (fg_ / sfh_fg): coefficients and data
          in, composite, gradient and -logL out, every step; host timers around each call,
          L2 flushed between calls
  templates_per_s : the 1,200-template GPU build (partial_cmd_smooth), CUDA events

`--impl reference` times the FP64 CPU restatement of the reference's fg! (the oracle)
on all host cores, same metric and configuration.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "starformationhistories.jl_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "logL+grad evals/s (fg!, one coefficient vector, 1200 templates x 60000 bins)"
UNIT = "evals/s"
WORKLOAD = "config2: 1200 templates, 200x300 Hess grid, 1e6 stars"
NBINS, NT = 60000, 1200


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


def _profile_value(key: str):
    """A figure `key: value` from the committed ncu summaries, else None."""
    pdir = os.path.join(ROOT, "profiles")
    for name in sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []:
        if not name.endswith(".md"):
            continue
        with open(os.path.join(pdir, name)) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":", 1)[1].strip().split()[0])
    return None


def _profile_traffic(kernel: str):
    """dram bytes per launch of `kernel` from the committed ncu summaries, else None."""
    pdir = os.path.join(ROOT, "profiles")
    for name in sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []:
        if not name.endswith(".md"):
            continue
        with open(os.path.join(pdir, name)) as f:
            for line in f:
                if line.startswith(f"dram_bytes_per_launch {kernel}:"):
                    return float(line.split(":", 1)[1].strip().split()[0])
    return None


class L2Flush:
    """Writes a device buffer of twice the L2 size on a stream. Called between timed
    iterations, outside their CUDA-event intervals, so that no iteration finds the
    previous one's inputs in L2 (the occupied-bin plan streams 66 MB, which would fit)."""

    def __init__(self, dev):
        import torch
        l2 = int(getattr(torch.cuda.get_device_properties(dev), "L2_cache_size", 0) or 0)
        self.nbytes = 2 * max(l2, 129 << 20)
        self.buf = torch.empty(self.nbytes // 4, dtype=torch.int32, device=dev)
        self.k = 0

    def __call__(self, stream):
        import torch
        self.k += 1
        with torch.cuda.stream(stream):
            self.buf.fill_(self.k)


def _timed_flushed(step, n, stream, flush):
    """Per-iteration CUDA-event times (ms) of n calls of step() on `stream`, with an L2
    flush before each, outside the intervals."""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(n)]
    with torch.cuda.stream(stream):
        for a, b in evs:
            flush(stream)
            a.record(stream)
            step()
            b.record(stream)
    evs[-1][1].synchronize()
    return [a.elapsed_time(b) for a, b in evs]


class Clocks:
    """nvidia-smi sampling during the timed region (200 ms period)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        self.f.close()
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    from sfhgpu.replicas import dist_env
    return dist_env()


def _barrier(world):
    from sfhgpu.replicas import barrier
    barrier(world)


def _max_over_ranks(world, x: float) -> float:
    from sfhgpu.replicas import max_over_ranks
    return max_over_ranks(world, x)


def _bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured"
    except Exception:  # noqa: BLE001
        return 1900.0, "fallback"


def run_batched(ctx, d_T, nbins, nt, r, data, M64, steps, warmup, B=4096, check=8):
    """Many coefficient vectors per call on the tensor cores (sfh_fg_batched_dev)."""
    import numpy as np
    import torch

    import sfhgpu
    L = sfhgpu.load()
    dev = torch.device("cuda", ctx.device)
    Hb = sfhgpu.Models.from_device(d_T.data_ptr(), nbins, nt, storage="bf16x2", ctx=ctx)
    rng = np.random.default_rng(7)
    R = r[None, :] * np.exp(0.3 * rng.standard_normal((B, nt)))  # chain states near r
    d_R = torch.tensor(R, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_L = torch.empty(B, dtype=torch.float64, device=dev)
    d_G = torch.empty((B, nt), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    args = (ctx.handle, Hb.handle, d_R.data_ptr(), B, d_n.data_ptr(), d_L.data_ptr(),
            d_G.data_ptr(), float(np.finfo(np.float64).eps))
    for _ in range(warmup):
        sfhgpu._lib.check(L.sfh_fg_batched_dev(*args), ctx.handle, "sfh_fg_batched_dev")
    ts = ctx.torch_stream()

    def call():
        sfhgpu._lib.check(L.sfh_fg_batched_dev(*args), ctx.handle, "sfh_fg_batched_dev")
    # L2 flushed before each call, outside its CUDA-event interval
    ms = float(np.mean(_timed_flushed(call, steps, ts, L2Flush(dev))))
    negL = d_L.cpu().numpy()
    # outputs for the accuracy check against the FP64 oracle, done in the CPU leg
    check_data = {"R": R[:check], "negL": negL[:check]}
    nst = float(data.sum())
    # algorithmic FLOPs: the two products C = R M^T and G = W M, 2 nbins nt B each, over
    # the bins the call needs (the occupied ones under an occupied-bin plan); the
    # digit-plane products of the exact composite and the hi/lo products of G are
    # implementation work and are not counted
    nocc, sparse, _ = Hb.occupied_info(d_n.data_ptr())
    nb_alg = nocc if sparse else nbins
    flops = 4.0 * nb_alg * nt * B
    peak, kind = _bf16_peak()
    Hb.free()
    return {
        "workload": f"{B} coefficient vectors x {nt} templates x {nbins} bins (one call)",
        "evals_per_s": B / (ms / 1e3), "ms_per_batch": ms, "B": B, "steps": steps,
        "composite": "exact digit planes (logL), BF16 hi/lo products for G = W M",
        "tensor_roofline": {"bound": "tensor", "achieved": flops / (ms / 1e3) / 1e12,
                            "peak": peak, "unit": "TFLOP/s",
                            "frac": flops / (ms / 1e3) / 1e12 / peak, "peak_source": kind,
                            "flops": "algorithmic: 4 bins nt B per call over the "
                                     f"{'occupied' if sparse else 'all'} bins ({nb_alg})",
                            "dense_equivalent_tflops": 4.0 * nbins * nt * B / (ms / 1e3) / 1e12},
        "occupied_bins": nocc if sparse else None,
        "_check": check_data,
    }


def run_hmc(ctx, d_T, w, nchains=1024, nwarmup=500, ntraj=1500, nleap=10, seed=20261205,
            d_model=None):
    """End-to-end hierarchical HMC (PowerLawMZR slope 0.5, GaussianDispersion 0.2) on the
    1,200-template grid: all chains advance together, one batched tensor-core evaluation
    per leapfrog substep, trajectories replayed from a captured CUDA graph.  The data are
    drawn from the exact templates d_T; the sampler uses d_model when given (emulated
    templates with exact fallback), d_T otherwise."""
    import numpy as np
    import torch

    import sfhgpu
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR, calculate_coeffs
    nbins, nt = w.nbins, w.ntempl
    la, mh = w.template_params
    src = d_T if d_model is None else d_model
    Hb = sfhgpu.Models.from_device(src.data_ptr(), nbins, nt, storage="bf16x2", ctx=ctx)
    rng = np.random.default_rng(seed)
    mzr, disp = PowerLawMZR(0.5, -1.0, 6.0), GaussianDispersion(0.2)
    R = np.exp(0.5 * rng.standard_normal(w.logAges.size))
    M = d_T.double()
    c = calculate_coeffs(mzr, disp, R, la, mh)
    R = R * (1e6 / float((M.T @ torch.as_tensor(c, device=M.device)).sum()))
    c = calculate_coeffs(mzr, disp, R, la, mh)
    data = rng.poisson((M.T @ torch.as_tensor(c, device=M.device)).cpu().numpy()).astype(float)
    del M
    torch.cuda.synchronize()
    l0 = ctx.launches
    t0 = time.perf_counter()
    out = sfhgpu.sample_sfh(Hb, data, la, mh, PowerLawMZR(0.45, -0.9, 6.0),
                            GaussianDispersion(0.25), R * 1.1, nsteps=ntraj, nchains=nchains,
                            nwarmup=nwarmup, nleap=nleap, step0=1e-3, seed=seed)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    launches = ctx.launches - l0
    Hb.free()
    substeps = nchains * (nwarmup + ntraj) * nleap
    na = w.logAges.size
    pm = out["mean"].mean(0)
    return {
        "workload": f"{nchains} chains x {nwarmup}+{ntraj} trajectories x {nleap} leapfrog "
                    f"steps, PowerLawMZR + GaussianDispersion over {nt} templates x {nbins} bins",
        "chain_gradient_evals_per_s": substeps / dt, "seconds": dt,
        "trajectories_per_s": nchains * (nwarmup + ntraj) / dt, "gpu_launches": launches,
        "accept_mean": float(np.mean(out["accept"])),
        "posterior_mean_alpha_MH0_sigma": [float(x) for x in pm[na:na + 3]],
        "truth_alpha_MH0_sigma": [0.5, -1.0, 0.2],
        "posterior_mean_abs_err": [float(abs(a - b)) for a, b in zip(pm[na:na + 3],
                                                                      [0.5, -1.0, 0.2])],
        "posterior_mean_R": [float(x) for x in pm[:na]],
        "note": "wall clock of sample_sfh (setup, graph capture, warmup and sampling); "
                "one batched gradient per leapfrog step (the start gradient is carried over)",
    }


def run_hmc_matched(ctx, d_T, w, nchains=1024, nwarmup=200, ndraw=10, nref=200,
                    seed=20261207):
    """The batched sampler against the plain single-chain path at matched posterior-mean
    error, measured on the config-5 model (PowerLawMZR + GaussianDispersion, 1,200
    templates, trajectories of 10 leapfrog steps).  Every run starts from the device
    fit_sfh MAP point with its inverse-Hessian diagonal as the starting metric, as
    sample_sfh(fit=...) does.  A reference posterior mean comes from a long batched run;
    then the batched run (nchains x ndraw draws after nwarmup) and one chain on the
    single-vector fg! with the same total number of draws.  Error: RMS over all variables
    of (mean - reference) / posterior sd.  Since the error of a mean falls as
    1/sqrt(draws), the single chain's time at the batched run's error is its time x
    (e_single / e_batched)^2.  Then the No-U-Turn sampler as the reference's sample_sfh
    runs it (the MLE point, the MAP inverse Hessian as a dense metric), timed on the
    same chains."""
    import numpy as np
    import torch

    import sfhgpu
    from sfhgpu.sampling import GaussianDispersion, PowerLawMZR, calculate_coeffs
    la, mh = w.template_params
    Hb = sfhgpu.Models.from_device(d_T.data_ptr(), w.nbins, w.ntempl, storage="bf16x2", ctx=ctx)
    rng = np.random.default_rng(seed)
    mzr, disp = PowerLawMZR(0.5, -1.0, 6.0), GaussianDispersion(0.2)
    R = np.exp(0.5 * rng.standard_normal(w.logAges.size))
    M = d_T.double()
    c = calculate_coeffs(mzr, disp, R, la, mh)
    R = R * (1e6 / float((M.T @ torch.as_tensor(c, device=M.device)).sum()))
    c = calculate_coeffs(mzr, disp, R, la, mh)
    data = rng.poisson((M.T @ torch.as_tensor(c, device=M.device)).cpu().numpy()).astype(float)
    del M
    Hf = sfhgpu.Models.from_device(d_T.data_ptr(), w.nbins, w.ntempl, storage="f32", ctx=ctx)
    t0 = time.perf_counter()
    fit = sfhgpu.fit_sfh(PowerLawMZR(0.45, -0.9, 6.0), GaussianDispersion(0.25), Hf, data, la, mh,
                         x0=R * 1.1)
    t_fit = time.perf_counter() - t0
    print(f"[hmc] fit {t_fit:.2f} s, MAP status {fit.map.result['status']}, "
          f"{fit.map.result['iterations']} iterations, |g| {fit.map.result['g_norm']:.2e}",
          file=sys.stderr, flush=True)
    Hf.free()

    def run(nch, nsteps, sd, sampler="hmc", nw=nwarmup, **kw):
        torch.cuda.synchronize()
        l0 = ctx.launches
        t0 = time.perf_counter()
        out = sfhgpu.sample_sfh(Hb, data, la, mh, nsteps=nsteps, nchains=nch, nwarmup=nw,
                                nleap=10, step0=0.05, seed=sd, fit=fit, sampler=sampler, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out["launches"] = ctx.launches - l0
        print(f"[hmc] {sampler} {nch} chains x {nsteps} draws: {dt:.2f} s, accept "
              f"{out['accept'].mean():.3f}", file=sys.stderr, flush=True)
        return out, dt

    ref, t_ref = run(nchains, nref, seed + 1)
    mref = ref["mean"].mean(0)
    sdref = np.sqrt(ref["var"].mean(0) + ref["mean"].var(0))
    bat, t_bat = run(nchains, ndraw, seed + 2)
    one, t_one = run(1, nchains * ndraw, seed + 3)
    nuts, t_nuts = run(nchains, 50, seed + 4, sampler="nuts", nw=50, max_depth=8)
    # the same sampler with the Laplace approximation of the posterior in the sampler's
    # space: chains from its mode (the MAP point) and its covariance as the dense metric
    # (curvature of log p by central differences of one batched gradient evaluation)
    t0 = time.perf_counter()
    cov = sfhgpu.laplace_metric(Hb, data, fit.map.theta, mzr=fit.map.MH_model,
                                disp=fit.map.disp_model, logAge=la, MH=mh)
    t_lap = time.perf_counter() - t0
    na = w.logAges.size
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nuts_l = sfhgpu.sample_sfh(Hb, data, la, mh, fit.map.MH_model, fit.map.disp_model,
                               np.asarray(fit.map.mu[:na], float), nsteps=50, nchains=nchains,
                               nwarmup=50, step0=0.05, seed=seed + 4, jitter=0.0,
                               sampler="nuts", max_depth=8, minv_dense=cov)
    torch.cuda.synchronize()
    t_nuts_l = time.perf_counter() - t0
    print(f"[hmc] nuts (Laplace metric at the MAP) {nchains} chains x 50 draws: "
          f"{t_nuts_l:.2f} s, accept {nuts_l['accept'].mean():.3f}, depth "
          f"{nuts_l['depth'].mean():.2f}", file=sys.stderr, flush=True)
    Hb.free()
    err = lambda mu: float(np.sqrt(np.mean(((mu - mref) / sdref) ** 2)))
    e_b, e_1 = err(bat["mean"].mean(0)), err(one["mean"][0])
    t_match = t_one * (e_1 / e_b) ** 2
    return {
        "workload": f"PowerLawMZR + GaussianDispersion over {w.ntempl} templates x {w.nbins} "
                    f"bins; trajectories of 10 leapfrog steps, {nwarmup} warmup trajectories "
                    "per chain; every run starts from the device fit_sfh MAP point",
        "map_fit_seconds": t_fit,
        "map_fit": {k: fit.map.result[k] for k in ("status", "iterations", "g_norm")},
        "reference": {"chains": nchains, "draws_per_chain": nref, "seconds": t_ref},
        "batched": {"chains": nchains, "draws_per_chain": ndraw, "seconds": t_bat,
                    "error": e_b, "accept": float(bat["accept"].mean())},
        "single_chain_plain": {"draws": nchains * ndraw, "seconds": t_one, "error": e_1,
                               "accept": float(one["accept"].mean())},
        "single_chain_seconds_at_batched_error": t_match,
        "speedup_at_matched_error": t_match / t_bat,
        "error": "RMS over the 43 variables of (posterior mean - reference) / posterior sd",
        "nuts": {"chains": nchains, "warmup_trees": 50, "draws_per_chain": 50,
                 "max_depth": 8, "seconds": t_nuts,
                 "trees_per_s": nchains * 100 / t_nuts,
                 "mean_depth": float(nuts["depth"].mean()),
                 "accept": float(nuts["accept"].mean()),
                 "divergent": int(nuts["divergent"].sum()),
                 "metric": "dense: the MAP inverse Hessian, from the MLE point (the "
                           "reference's sample_sfh); the step adapted over the warmup trees"},
        "nuts_laplace_metric": {
            "chains": nchains, "warmup_trees": 50, "draws_per_chain": 50, "max_depth": 8,
            "metric_seconds": t_lap, "seconds": t_nuts_l,
            "trees_per_s": nchains * 100 / t_nuts_l,
            "mean_depth": float(nuts_l["depth"].mean()),
            "accept": float(nuts_l["accept"].mean()),
            "divergent": int(nuts_l["divergent"].sum()),
            "error_vs_reference": err(nuts_l["mean"].mean(0)),
            "metric": "dense: the Laplace covariance at the MAP point (laplace_metric), "
                      "chains from the MAP point; the step adapted over the warmup trees"},
    }


def run_ragged(ctx, steps=50, warmup=5, check=2):
    """256 independent galaxies with uneven Hess grids (50-300 bins per axis) and
    isochrone lengths (100-2,000 points): one ragged template build, then fg! over all
    galaxies per call (sfh_fg_ragged_dev)."""
    import numpy as np
    import torch

    import sfhgpu
    from sfhgpu import synthetic as S
    dev = torch.device("cuda", ctx.device)
    gals = S.ragged()
    m, mags, offs, lens, dm, edges = S.ragged_isochrones(gals)
    d_m, d_mags = torch.as_tensor(m, device=dev), torch.as_tensor(mags, device=dev)
    args = (d_m, d_mags, offs, lens, 1, (0, 1), S.error_models(), S.completeness_models(),
            S.imf(), dm, 1.0, edges)
    out, toff = sfhgpu.partial_cmd_smooth_ragged(*args, ctx=ctx)  # warm-up, sizes the output
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sfhgpu.partial_cmd_smooth_ragged(*args, out=out, ctx=ctx)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    nt = np.array([g.ntempl for g in gals])
    nb = np.array([g.nbins for g in gals])
    gal = sfhgpu.Galaxies(out, nb, nt, ctx=ctx)
    # per-galaxy coefficients exp(N(0,1)) scaled to 1e4 stars, Poisson data
    rng = np.random.default_rng(11)
    r = np.exp(rng.standard_normal(int(nt.sum())))
    _, _, comp = sfhgpu.fg_ragged(gal, r, np.zeros(int(nb.sum())), want_logl=False,
                                  want_grad=False)
    comp = comp.cpu().numpy()
    for g in range(len(gals)):
        b0, b1 = gal.bin_offsets[g], gal.bin_offsets[g + 1]
        t0_, t1_ = gal.templ_offsets[g], gal.templ_offsets[g + 1]
        r[t0_:t1_] *= 1e4 / max(comp[b0:b1].sum(), 1e-300)
    _, _, comp = sfhgpu.fg_ragged(gal, r, np.zeros(int(nb.sum())), want_logl=False,
                                  want_grad=False)
    data = rng.poisson(np.maximum(comp.cpu().numpy(), 0)).astype(float)
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_c = torch.empty_like(d_n)
    d_G = torch.empty_like(d_r)
    d_L = torch.empty(len(gals), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    L = sfhgpu.load()
    eps = float(np.finfo(np.float64).eps)
    call = (ctx.handle, gal.handle, d_r.data_ptr(), d_n.data_ptr(), d_c.data_ptr(),
            d_G.data_ptr(), d_L.data_ptr(), eps)
    for _ in range(warmup):
        sfhgpu._lib.check(L.sfh_fg_ragged_dev(*call), ctx.handle, "fg_ragged")
    ts = ctx.torch_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ts)
    for _ in range(steps):
        sfhgpu._lib.check(L.sfh_fg_ragged_dev(*call), ctx.handle, "fg_ragged")
    e1.record(ts)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # outputs of the largest galaxies for the accuracy check against the FP64 oracle,
    # done in the CPU leg
    negL, G = d_L.cpu().numpy(), d_G.cpu().numpy()
    check_data = []
    for g in np.argsort(-nb)[:check]:
        mo = int(sum(nb[:g] * nt[:g]))
        b0, b1 = gal.bin_offsets[g], gal.bin_offsets[g + 1]
        t0_, t1_ = gal.templ_offsets[g], gal.templ_offsets[g + 1]
        Mg = out[mo:mo + int(nb[g] * nt[g])].cpu().numpy().reshape(int(nt[g]), int(nb[g])).T
        check_data.append((Mg, r[t0_:t1_].copy(), data[b0:b1].copy(), float(negL[g]),
                           G[t0_:t1_].copy()))
    # galaxies with <= 32 templates take the fused pass (M read once); larger ones read
    # M twice (composite pass, then the gradient pass)
    reads = np.where(nt <= 32, 1, 2)
    alg_bytes = (4 * float((reads * nb * nt).sum()) + 16 * float(nb.sum())
                 + 16 * float(nt.sum()))
    peak, kind = _peaks()
    gal.free()
    return {
        "workload": f"{len(gals)} galaxies, grids 50-300 bins per axis ({int(nb.sum())} bins), "
                    f"isochrones 100-2000 points, {int(nt.sum())} templates",
        "templates_per_s": float(nt.sum()) / build_s, "template_build_s": build_s,
        "fg_calls_per_s": 1e3 / ms, "galaxy_evals_per_s": len(gals) * 1e3 / ms,
        "ms_per_call": ms,
        "roofline": {"bound": "hbm", "achieved": alg_bytes / (ms * 1e-3) / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": alg_bytes / (ms * 1e-3) / 1e9 / peak,
                     "peak_source": kind, "algorithmic_bytes_per_call": alg_bytes},
        "_check": check_data,
    }


def run_emulator(ctx, w, n_train=150_000, n_val=8192, steps=60000, cells=(32, 4, 1),
                 trust_cells=None, nreq=1200):
    """Learned template emulator for one galaxy at a known distance: theta = (log age,
    [M/H]) over the whole production grid's box with the distance modulus within 0.05 mag
    of the galaxy's.  Per-cell PCA bases (64 components of sqrt templates) and per-cell MLPs
    3-256-256-64 trained on templates the GPU partial_cmd_smooth generates at random; a
    trust map (on the basis cells unless trust_cells is given) keeps each cell's worst
    validation deviance.  Scored
    by Poisson deviance per star against exact templates (tolerance 1e-3) on the 1,200
    templates of the production grid (the requests a fit of that galaxy makes) and on
    random requests; routed = emulated where trusted, exact elsewhere."""
    import numpy as np
    import torch

    from sfhgpu.emulator import SyntheticGenerator, TemplateEmulator, group_segments
    gen = SyntheticGenerator(w.xedges, w.yedges, ctx=ctx)
    bounds = ((6.6, 10.1), (-2.5, 0.3), (w.dmod - 0.05, w.dmod + 0.05))
    em = TemplateEmulator(gen.nbins, ncomp=64, hidden=(256, 256), tol=1e-3, bounds=bounds,
                          basis_cells=cells, trust_cells=trust_cells, ctx=ctx)
    t0 = time.perf_counter()
    rep = em.fit(gen, n_train=n_train, n_val=n_val, steps=steps, lr=1e-3, batch_per_cell=32)
    fit_s = time.perf_counter() - t0
    la, mh = w.template_params
    th_grid = np.stack([la, mh, np.full(la.size, w.dmod)], 1)
    th_rand = em.sample_theta(nreq, np.random.default_rng(5))

    def timed(f, reps=5):
        f()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            r = f()
        torch.cuda.synchronize()
        return r, (time.perf_counter() - t0) / reps

    out = {}
    for name, th in (("grid", th_grid), ("random", th_rand)):
        exact, t_exact = timed(lambda: gen(th), reps=2)
        emul, t_emul = timed(lambda: em.predict(th))
        dev = em.score(exact, emul)
        trusted = em.trusted(th)
        (routed, used), t_routed = timed(lambda: em.templates(th, gen), reps=2)
        assert np.array_equal(used, trusted)
        dr = em.score(exact, routed)
        out[name] = {
            "requests": int(th.shape[0]),
            "frac_within_1e-3": float(np.mean(dev <= 1e-3)),
            "frac_within_1e-2": float(np.mean(dev <= 1e-2)),
            "deviance_median": float(np.median(dev)),
            "trusted_frac": float(np.mean(trusted)),
            "trusted_within_1e-3": float(np.mean(dev[trusted] <= 1e-3)) if trusted.any() else None,
            "routed_deviance_max": float(dr.max()),
            "emulated_templates_per_s": th.shape[0] / t_emul,
            "exact_templates_per_s": th.shape[0] / t_exact,
            "routed_templates_per_s": th.shape[0] / t_routed,
            "routed_speedup_vs_exact": t_exact / t_routed,
        }
        del exact, emul, routed

    # the reconstruction kernel alone (cell segments; each segment reads its cell's basis once)
    coef = em.coefficients(th_grid)
    rows, seg = group_segments(em.group_of(th_grid))
    d_rows = torch.as_tensor(rows, device=coef.device)
    d_seg = torch.as_tensor(seg, device=coef.device)
    B = th_grid.shape[0]
    buf = torch.empty((B, em.nbins), dtype=torch.float32, device=coef.device)
    import sfhgpu
    L = sfhgpu.load()
    peak, peak_src = _peaks()
    s = ctx.torch_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def recon():
        L.sfh_emu_reconstruct_groups(ctx.handle, coef.data_ptr(), d_rows.data_ptr(),
                                     d_seg.data_ptr(), seg.shape[0], em.ngroups,
                                     em.basis.data_ptr(), em.offset.data_ptr(), em.K, em.nbins,
                                     B, em.mode, buf.data_ptr())
    torch.cuda.synchronize()
    for _ in range(3):
        recon()
    e0.record(s)
    for _ in range(20):
        recon()
    e1.record(s)
    torch.cuda.synchronize()
    t_rec = e0.elapsed_time(e1) / 20 * 1e-3
    rec_bytes = 4.0 * em.nbins * (seg.shape[0] * (em.K + 1) + B)
    run_emulator.last = em
    return {
        "workload": f"one galaxy at distance modulus {w.dmod} (+-0.05): {n_train} training "
                    f"templates on the 200x300 grid, theta = (log age U[6.6,10.1], [M/H] "
                    f"U[-2.5,0.3], dmod); {int(np.prod(cells))} basis cells {cells}, PCA 64 of "
                    f"sqrt templates, MLP 3-256-256-64 per cell trained for {steps} steps; "
                    f"trust map on {trust_cells or cells} cells from {n_val} validation "
                    f"templates; requests: the {B} templates of "
                    f"the production grid and {nreq} random theta",
        "fit_seconds": fit_s, "generate_seconds": rep.generate_seconds,
        "pca_seconds": rep.pca_seconds, "train_seconds": rep.train_seconds,
        "final_loss": rep.final_loss, "val_deviance_quantiles": rep.val_deviance_quantiles,
        "val_frac_within_1e-3": rep.val_frac_within_tol,
        "trusted_cell_fraction": rep.trusted_cell_fraction,
        "grid_requests": out["grid"], "random_requests": out["random"],
        "reconstruct_roofline": {
            "kernel": "k_recon_groups", "bound": "hbm", "segments": int(seg.shape[0]),
            "ms": t_rec * 1e3, "achieved": rec_bytes / t_rec / 1e9,
            "peak": peak, "peak_source": peak_src, "unit": "GB/s",
            "frac": rec_bytes / t_rec / 1e9 / peak,
            "bytes": "4 nbins (segments (K + 1) + B): each segment's basis and offset read "
                     "once, every template written once"},
    }


def run_fit(H, data, g_abstol=1e-3):
    """fit_templates_fast / fit_templates on the headline templates: the device BFGS driver
    (host arrays in, coefficients out) against scipy's BFGS looping over the host-array
    fg! (the shape of the reference's Optim loop), both from x0 = ones, renormalised."""
    import numpy as np

    import sfhgpu
    x0 = np.ones(H.nt)
    sfhgpu.fit_templates_fast(H, data, x0=x0, g_abstol=g_abstol, maxiter=3)  # warm
    t0 = time.perf_counter()
    xd, rd = sfhgpu.fit_templates_fast(H, data, x0=x0, g_abstol=g_abstol, maxiter=3000)
    td = time.perf_counter() - t0
    t0 = time.perf_counter()
    res = sfhgpu.fit_templates(H, data, x0=x0, gtol=g_abstol, maxiter=3000)
    tm = time.perf_counter() - t0
    t0 = time.perf_counter()
    xs, rs = sfhgpu.fit_templates_fast(H, data, x0=x0, g_abstol=g_abstol, maxiter=3000,
                                       method="scipy")
    ts = time.perf_counter() - t0
    big = xs > 1e-3 * xs.max()
    return {
        "g_abstol": g_abstol, "x0": "ones, renormalised (renormalize_x0)",
        "device": {"seconds": td, "nfev": rd.nfev, "nit": rd.nit, "status": rd.message,
                   "ms_per_eval": td / rd.nfev * 1e3, "f": rd.fun, "graph": rd.graph},
        "scipy_host_loop": {"seconds": ts, "nfev": int(rs.nfev), "nit": int(rs.nit),
                            "f": float(rs.fun), "ms_per_eval": ts / rs.nfev * 1e3},
        "speedup_vs_scipy_host_loop": ts / td,
        "f_device_minus_scipy": float(rd.fun - rs.fun),
        "coeff_rel_diff_max": float(np.max(np.abs(xd[big] / xs[big] - 1.0))),
        "fit_templates_map_mle": {"seconds": tm,
                                  "nfev": res.map.result.nfev + res.mle.result.nfev,
                                  "status": [res.map.result.message, res.mle.result.message]},
    }


def run_extras(ctx, w, cpu=True, ntempl=60, nstars=10_000_000):
    """The rows beside the headline path, each timed on the GPU with CUDA events and, when
    `cpu`, beside the oracle (or a numpy port) on a bounded sample:
    binary_hess (RandomBinaryPairs) for `ntempl` templates of the production grid, bin_cmd
    of `nstars` catalogue-precision stars on the production grid and on a 100 x 100 grid,
    and model_cmd of `nstars` three-filter stars."""
    import ctypes as C

    import numpy as np
    import torch

    import sfhgpu
    from sfhgpu import synthetic as S
    L = sfhgpu.load()
    dev = torch.device("cuda", 0)
    out = {}

    def ev_time(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ctx.torch_stream()):
            e0.record(ctx.torch_stream())
            for _ in range(reps):
                fn()
            e1.record(ctx.torch_stream())
        e1.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3  # seconds

    # ---- binary_hess for ntempl templates (host preprocessing of the pair points once)
    m_ini, mags, offs, lens = S.isochrone_batch(w)
    pts = [sfhgpu.binary_points(m_ini[o:o + n], list(mags[:, o:o + n]), 1, (0, 1), w.dmod,
                                (w.xedges, w.yedges)) for o, n in list(zip(offs, lens))[:ntempl]]
    md = np.concatenate([p[0] for p in pts])
    gd = np.ascontiguousarray(np.concatenate([p[1] for p in pts], axis=1))
    ln = np.array([p[0].size for p in pts], dtype=np.int32)
    of = np.concatenate([[0], np.cumsum(ln)[:-1]]).astype(np.int64)
    d_m, d_g = torch.tensor(md, device=dev), torch.tensor(gd, device=dev)
    imf = S.imf()
    nx, ny = w.grid
    buf = torch.empty((len(pts), nx * ny), dtype=torch.float32, device=dev)

    def binary():
        sfhgpu.binary_hess_batch(d_m, d_g, of, ln, 1, (0, 1), S.error_models(),
                                 S.completeness_models(), imf, w.normalize_value,
                                 (w.xedges, w.yedges), out=buf)
    t = ev_time(binary, 3)
    pairs = float(np.sum(ln.astype(np.float64) * (ln - 1) / 2))
    out["binary_hess"] = {"templates": len(pts), "seconds": t, "templates_per_s": len(pts) / t,
                          "pairs_per_s": pairs / t, "mean_points_per_template": float(ln.mean())}

    # ---- bin_cmd: catalogue-precision stars (3 decimals: many on edges)
    rng = np.random.default_rng(5)
    x = np.round(rng.normal(0.8, 0.5, nstars), 3)
    y = np.round(rng.uniform(float(w.yedges[0]), float(w.yedges[-1]), nstars), 3)
    d_x, d_y = torch.tensor(x, device=dev), torch.tensor(y, device=dev)
    for name, (ex, ey) in (("production_grid", (w.xedges, w.yedges)),
                           ("grid_100x100", (sfhgpu.julia_range(-1.0, 3.0, 101),
                                             sfhgpu.julia_range(float(w.yedges[0]),
                                                                float(w.yedges[-1]), 101)))):
        ex, ey = np.ascontiguousarray(ex, dtype=np.float64), np.ascontiguousarray(ey, dtype=np.float64)
        d_ex, d_ey = torch.tensor(ex, device=dev), torch.tensor(ey, device=dev)
        gx, gy = ex.size - 1, ey.size - 1
        d_h = torch.empty(gx * gy, dtype=torch.float64, device=dev)

        def bc():
            rc = L.sfh_bin_cmd_dev(ctx.handle, d_x.data_ptr(), d_y.data_ptr(), None, nstars,
                                   d_ex.data_ptr(), gx, d_ey.data_ptr(), gy, d_h.data_ptr())
            if rc:
                sfhgpu._lib.check(rc, ctx.handle, "sfh_bin_cmd_dev")
        t = ev_time(bc, 20)
        t0 = time.perf_counter()
        h = sfhgpu.bin_cmd(x, y, edges=(ex, ey)).weights
        te = time.perf_counter() - t0
        leg = {"bins": gx * gy, "stars": nstars, "device_seconds": t,
               "stars_per_s": nstars / t, "e2e_stars_per_s": nstars / te,
               "achieved_gbs": nstars * 16 / t / 1e9}
        if cpu:
            import oracle as O
            ns = 2_000_000
            t0 = time.perf_counter()
            ref = O.bin_cmd(x[:ns], y[:ns], None, ex, ey)
            leg["cpu_baseline"] = {"stars_per_s": ns / (time.perf_counter() - t0), "cores": 1,
                                   "kind": "port", "sample": f"{ns} stars (oracle, 1 thread)"}
            hs = sfhgpu.bin_cmd(x[:ns], y[:ns], edges=(ex, ey)).weights
            leg["bit_exact_vs_oracle"] = bool(np.array_equal(hs, ref))
        out["bin_cmd_" + name] = leg

    # ---- model_cmd: three filters
    m3 = np.ascontiguousarray(rng.uniform(22.0, 30.0, (nstars, 3)))
    sig = np.ascontiguousarray(0.01 + 0.3 * np.exp((m3 - 28.0) / 1.2))
    prob = np.ascontiguousarray(np.prod(1.0 / (1.0 + np.exp((m3 - 28.0) / 0.3)), axis=1))
    d_m3, d_sig, d_p = (torch.tensor(a, device=dev) for a in (m3, sig, prob))
    d_out = torch.empty_like(d_m3)
    d_idx = torch.empty(nstars, dtype=torch.int64, device=dev)
    nout = C.c_int64()

    def mc():
        rc = L.sfh_model_cmd_dev(ctx.handle, d_m3.data_ptr(), d_sig.data_ptr(), None,
                                 d_p.data_ptr(), nstars, 3, 7, d_out.data_ptr(),
                                 d_idx.data_ptr(), C.byref(nout))
        if rc:
            sfhgpu._lib.check(rc, ctx.handle, "sfh_model_cmd_dev")
    t = ev_time(mc, 10)
    leg = {"stars": nstars, "kept": int(nout.value), "device_seconds": t,
           "stars_per_s": nstars / t, "note": "includes the synchronisation that reads the count"}
    if cpu:
        ns = 2_000_000
        g = np.random.default_rng(1)
        t0 = time.perf_counter()
        keep = g.random(ns) <= prob[:ns]
        _ = m3[:ns][keep] + g.standard_normal((int(keep.sum()), 3)) * sig[:ns][keep]
        leg["cpu_baseline"] = {"stars_per_s": ns / (time.perf_counter() - t0), "cores": 1,
                               "kind": "port", "sample": f"{ns} stars (numpy, 1 thread)"}
    out["model_cmd"] = leg
    return out


def oracle_checks(batched, ragged, M64, r, data, neglogl):
    """Accuracy against the FP64 oracle on the same stored templates (CPU leg): the plain
    fg!'s -logL, and the stashed outputs of the batched and ragged legs (the stash is
    removed).  Returns the plain path's figures."""
    import numpy as np
    import torch

    import oracle as O
    thr = os.cpu_count() or 1
    O.set_threads(thr)
    nst = float(data.sum())
    v_ref, _, _ = O.fg(r, M64, data)
    plain = {"dlogL_per_1e4_stars_vs_oracle": abs(neglogl - v_ref) / (nst / 1e4),
             "negLogL_oracle": v_ref}
    if batched and "_check" in batched:
        c = batched.pop("_check")
        # FP64 oracle on the stored FP32 templates and the exact FP64 coefficient vectors
        ref_f, _ = O.fg_batched(c["R"], M64, data, nthreads=thr, want_g=False)
        batched["dlogL_per_1e4_stars_vs_oracle"] = float(
            np.max(np.abs(c["negL"] - ref_f)) / (nst / 1e4))
        batched["vectors_checked"] = int(len(c["negL"]))
    if ragged and "_check" in ragged:
        err_l, err_g = 0.0, 0.0
        for Mg, rg, ng, negl, Gg in ragged.pop("_check"):
            Mg = np.asfortranarray(Mg, dtype=np.float64)
            v, Gr, w = O.fg(rg, Mg, ng)
            err_l = max(err_l, abs(negl - v) / max(1.0, ng.sum() / 1e4))
            err_g = max(err_g, float(np.max(np.abs(Gg - Gr) /
                                            (np.abs(Mg).T @ (np.abs(w) + np.abs(1 - w)) + 1e-300))))
        ragged["dlogL_per_1e4_stars_vs_oracle"] = err_l
        ragged["grad_err_rel_scale_vs_oracle"] = err_g
    return plain


def template_checks(w, m_ini, mags, offs, lens, M32, nsample=8):
    """FP32 GPU templates of the timed build against the FP64 oracle's partial_cmd_smooth on
    `nsample` templates spread over the grid (a spawn process pool): the worst per-bin error
    normalised by the tolerance 1e-5 |ref| + 1e-6 max(ref) (<= 1 passes) and the largest
    relative error over bins above 1e-3 of the template's maximum."""
    import numpy as np

    import oracle as O
    from sfhgpu import synthetic as S
    nx, ny = w.grid
    ex = (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx)
    ey = (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny)
    err = [(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    com = [(c.A, c.m50, c.rho) for c in S.completeness_models()]
    idx = np.linspace(0, w.ntempl - 1, nsample).astype(int)
    jobs = [(m_ini[offs[t]:offs[t] + lens[t]], mags[:, offs[t]:offs[t] + lens[t]], err, com, 1,
             (0, 1), w.dmod, 1.0, ex, ey) for t in idx]
    t0 = time.perf_counter()
    refs = O.partial_cmd_smooth_many(jobs)
    worst, relmax = 0.0, 0.0
    for k, t in enumerate(idx):
        R = refs[k]
        G = M32[t].reshape(ny, nx).T.astype(np.float64)
        e = np.abs(G - R)
        worst = max(worst, float(np.max(e / np.maximum(1e-5 * np.abs(R) + 1e-6 * np.abs(R).max(),
                                                       1e-300))))
        big = np.abs(R) > 1e-3 * np.abs(R).max()
        relmax = max(relmax, float(np.max(e[big] / np.abs(R[big]))))
    return {"templates_checked": int(idx.size), "max_err_over_tolerance": worst,
            "max_rel_err_bins_above_1e-3_of_max": relmax,
            "tolerance": "1e-5 |ref| + 1e-6 max(ref) per bin", "oracle_seconds":
            time.perf_counter() - t0}


def cpu_fg_baseline(M64, r, data, budget_s=10.0, threads=None):
    """The oracle's fg! (FP64, OpenMP over bins/templates) on a bounded number of evals."""
    import numpy as np
    import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    O.fg(r, M64, data)  # warm
    t0 = time.perf_counter()
    O.fg(r, M64, data)
    one = time.perf_counter() - t0
    n = max(2, min(500, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(n):
        O.fg(r, M64, data)
    dt = time.perf_counter() - t0
    del np
    return n / dt, threads, n, dt


def cpu_template_baseline(w, budget_s=8.0):
    """The oracle's partial_cmd_smooth (FP64, one thread) on a sample of templates."""
    import oracle as O
    from sfhgpu import synthetic as S
    m_ini, mags, offs, lens = S.isochrone_batch(w)
    nx, ny = w.grid
    oimf = O.kroupa2001()
    E = [O.ErrModel(e.a, e.b, e.c, e.d, e.cap) for e in S.error_models()]
    Cm = [O.ComplModel(c.A, c.m50, c.rho) for c in S.completeness_models()]
    ex = (w.xedges[0], (w.xedges[-1] - w.xedges[0]) / nx, nx)
    ey = (w.yedges[0], (w.yedges[-1] - w.yedges[0]) / ny, ny)
    # sample templates spread over the grid of ages/metallicities
    order = list(range(0, w.ntempl, max(1, w.ntempl // 16)))
    done, t0 = 0, time.perf_counter()
    for t in order:
        sl = slice(offs[t], offs[t] + lens[t])
        O.partial_cmd_smooth(m_ini[sl], mags[:, sl], E, Cm, 1, (0, 1), oimf, w.dmod, 1.0,
                             O.imf_mean(oimf), ex, ey)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return done / dt, done, dt


def run_reference(args):
    """`--impl reference`: the FP64 CPU restatement (oracle) of fg! on all host cores."""
    import numpy as np
    world, rank, _ = _dist()
    if rank != 0:
        return
    rng = np.random.default_rng(20261203)
    # fg! time does not depend on template values (dense FP64 gemv + gemvᵀ): a seeded
    # matrix of the workload's shape stands in for the 1,200 GPU-built templates.
    M64 = np.asfortranarray(rng.random((NBINS, NT)) * 1e-4)
    r = np.exp(rng.standard_normal(NT))
    r *= 1e6 / (M64 @ r).sum()
    data = rng.poisson(M64 @ r).astype(np.float64)
    import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    for _ in range(max(1, args.warmup)):
        O.fg(r, M64, data)
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    one = None
    done = 0
    for i in range(steps):
        O.fg(r, M64, data)
        done += 1
        if i == 0:
            one = time.perf_counter() - t0
        if time.perf_counter() - t0 > args.reference_budget_s:
            break
    dt = time.perf_counter() - t0
    v = done / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * dt / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "nbins": NBINS, "ntempl": NT},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{done} fg! evals (bounded to ~{args.reference_budget_s:.0f} s;"
                                   f" first eval {1e3 * (one or 0):.1f} ms)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes as C

    import numpy as np
    import torch

    import sfhgpu
    from sfhgpu import synthetic as S
    from sfhgpu.emulator import SyntheticGenerator

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = sfhgpu.Context(local)
    L = sfhgpu.load()
    tstream = ctx.torch_stream()
    w = S.config2()
    if args.ntempl != NT:
        # profiling case: the first ntempl templates of the production grid
        nages = max(1, args.ntempl // w.MHs.size)
        w.logAges = w.logAges[:nages]
        w.name = f"config2 grid, {w.ntempl} templates (profiling case)"
    nx, ny = w.grid
    NTW = w.ntempl

    # ---- template build (partial_cmd_smooth on the GPU), templates/s
    m_ini, mags, offs, lens = S.isochrone_batch(w)
    d_m = torch.tensor(m_ini, device=dev)
    d_mags = torch.tensor(mags, device=dev)
    torch.cuda.synchronize()
    d_T = torch.empty((w.ntempl, nx * ny), dtype=torch.float32, device=dev)

    def build():
        sfhgpu.partial_cmd_smooth_batch(d_m, d_mags, offs, lens, 1, (0, 1), S.error_models(),
                                        S.completeness_models(), S.imf(), w.dmod, 1.0,
                                        (w.xedges, w.yedges), out=d_T, ctx=ctx)

    build()  # warm-up (also allocates scratch)
    nbuild = 3
    with torch.cuda.stream(tstream):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(tstream)
        for _ in range(nbuild):
            build()
        e1.record(tstream)
    e1.synchronize()
    build_ms = e0.elapsed_time(e1) / nbuild
    templates_per_s = w.ntempl / (build_ms / 1e3)
    # work of the build in its own unit: bin updates (stamp windows clipped to the grid,
    # counted by the host mirror on 48 templates spread over the grid, scaled to all)
    from sfhgpu.templates import partial_cmd_smooth_stars, stamp_bin_updates
    la, mh = w.template_params
    pick = np.linspace(0, w.ntempl - 1, 48).astype(int)
    upd = 0
    for t in pick:
        mi, mg = S.isochrone(la[t], mh[t], w.n_iso)
        xs_, ys_, sx_, sy_, _, cov_, e_ = partial_cmd_smooth_stars(
            mi, list(mg), S.error_funcs(), 1, (0, 1), S.imf(), S.completeness_funcs(),
            dmod=w.dmod, edges=(w.xedges, w.yedges))
        upd += int(stamp_bin_updates(xs_, ys_, sx_, sy_, cov_, e_).sum())
    bin_updates = upd * w.ntempl / pick.size

    # ---- template matrix handle (FP32 storage) and observed data
    H = sfhgpu.Models.from_device(d_T.data_ptr(), NBINS, NTW, storage="f32", ctx=ctx)
    M32 = d_T.cpu().numpy()          # (nt, nbins) row-major == (nbins, nt) column-major
    M64 = np.asfortranarray(M32.T.astype(np.float64))
    r, data = S.observed(M64, w.n_stars, seed=w.seed)
    d_r = torch.tensor(r, device=dev)
    d_n = torch.tensor(data, device=dev)
    d_c = torch.empty(NBINS, dtype=torch.float64, device=dev)
    d_G = torch.empty(NTW, dtype=torch.float64, device=dev)
    d_L = torch.empty(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    eps = float(np.finfo(np.float64).eps)

    # launch plan picked by the library's autotuner on this matrix and these inputs
    H.set_occupied(args.occupied)
    tuned = ({"plan": [None, None, None], "ms": None} if args.no_autotune
             else H.autotune(r, data, iters=10))
    if args.fg_path != "auto":
        H.set_path(args.fg_path)
    if args.onepass_variant:
        # pins the one-pass variant (profiling runs, where timings under the profiler would
        # steer the autotuner): bins,ctas_per_sm,schedule,boxes_per_copy
        b, c, sch, rb = args.onepass_variant.split(",")
        H.set_onepass_tile(int(b))
        H.set_onepass_ctas(int(c))
        H.set_onepass_schedule(sch)
        H.set_onepass_run(int(rb))

    def step():
        rc = L.sfh_fg_dev(ctx.handle, H.handle, d_r.data_ptr(), d_n.data_ptr(), d_c.data_ptr(),
                          d_G.data_ptr(), d_L.data_ptr(), eps)
        if rc:
            sfhgpu._lib.check(rc, ctx.handle, "sfh_fg_dev")

    flush = L2Flush(dev)
    for _ in range(args.warmup):
        flush(tstream)
        step()
    ctx.synchronize()
    clocks = Clocks(local)
    _barrier(world)
    torch.cuda.synchronize()
    launches0 = ctx.launches
    clocks.start()
    time.sleep(0.25)  # let the sampler take its first reading under load
    step_ms = _timed_flushed(step, args.steps, tstream, flush)
    torch.cuda.synchronize()
    clk = clocks.stop()
    _barrier(world)
    launches = ctx.launches - launches0
    ms = _max_over_ranks(world, float(sum(step_ms)))
    value = world * args.steps / (ms / 1e3)
    neglogl = float(d_L.item())
    nocc, occ_sparse, occ_build_ms = H.occupied_info(d_n.data_ptr())
    nsm = torch.cuda.get_device_properties(0).multi_processor_count

    def kernel_times():
        kms = (C.c_double * 4)()
        sfhgpu._lib.check(L.sfh_fg_kernel_times(ctx.handle, H.handle, d_r.data_ptr(),
                                                d_n.data_ptr(), d_c.data_ptr(), d_G.data_ptr(),
                                                d_L.data_ptr(), eps, 50, kms),
                          ctx.handle, "sfh_fg_kernel_times")
        return kms

    # ---- the same evaluations on the dense kernel (every bin's template row streamed)
    occupied = None
    if occ_sparse and args.occupied == "auto":
        H.set_occupied("off")
        for _ in range(args.warmup):
            step()
        nd = min(args.steps, 1000)
        dense_step_ms = _timed_flushed(step, nd, tstream, flush)
        dense_ms = float(np.mean(dense_step_ms))
        dkms = [dense_ms] if H.path == "onepass" else kernel_times()
        dense_alg = NBINS * NTW * 4 + NTW * 8 + NBINS * 8 * 2 + 2 * nsm * NTW * 8 + NTW * 8
        dpeak, _ = _peaks()
        H.set_occupied("auto")
        for _ in range(args.warmup):  # a new plan for the timed data (built outside timing)
            step()
        ctx.synchronize()
        occupied = {
            "occupied_bins": nocc, "fraction": nocc / NBINS, "plan_build_ms": occ_build_ms,
            "dense_evals_per_s": world / (dense_ms / 1e3), "dense_ms_per_eval": dense_ms,
            "speedup_vs_dense": value / (world / (dense_ms / 1e3)),
            "dense_kernel_ms": dkms[0],
            "dense_roofline_frac": dense_alg / (dkms[0] * 1e-3) / 1e9 / dpeak,
            "note": "fg! with G needs the composite only where n > 0; empty bins enter "
                    "through FP64 template column sums (sfh_models_set_occupied)",
        }

    # ---- per-kernel times (CUDA events) for the roofline of the dominant kernel: on the
    # one-pass paths a step is one launch of the one kernel, so its average launch duration
    # is the timed region's mean step time (L2 flushed before each); the two-pass path
    # times its kernels separately (sfh_fg_kernel_times)
    kms = list(kernel_times())
    kms_back_to_back = list(kms)
    path = H.path
    if path == "onepass":
        kms[0] = float(np.mean(step_ms))
    if path == "onepass" and occ_sparse:
        # the one-pass kernel on the occupied-bin plan: the occupied bins' template rows
        # once, r, n and the composite of every bin (the empty ones are checked and set to
        # w = 1), the per-SM partials, G and the column sums over the empty bins
        names = ["k_fg_onepass_occupied", "(fused into the one-pass kernel)",
                 "(fused: grid reduction)", "(none)"]
        alg = [nocc * NTW * 4 + NTW * 8 + NBINS * 8 * 2 + 2 * nsm * NTW * 8 + 2 * NTW * 8, 0, 0, 0]
        alg_eval = nocc * NTW * 4 + NTW * 8 * 3 + NBINS * 8 * 2
    elif path == "onepass":
        # [0] the one-pass kernel (M once, r, n, composite out, G and -logL through
        # per-SM partials and an in-kernel grid reduction); slots [1]-[3] stay empty.
        names = ["k_fg_onepass", "(fused into the one-pass kernel)", "(fused: grid reduction)",
                 "(none)"]
        alg = [NBINS * NTW * 4 + NTW * 8 + NBINS * 8 * 2 + 2 * nsm * NTW * 8 + NTW * 8, 0, 0, 0]
        alg_eval = NBINS * NTW * 4 + NTW * 8 * 2 + NBINS * 8 * 2  # M once, r, n, composite, G
    else:
        # FP32 storage runs two fused kernels: [0] pass 1 (m, logL, w), [2] pass 2 (G);
        # slots [1] and [3] stay empty.
        names = ["k_fg_pass1_f32", "(fused into pass 1)", "k_fg_pass2_f32", "(fused into pass 2)"]
        alg = [NBINS * NTW * 4 + NTW * 8 + NBINS * 8,    # M, r, m
               NBINS * 8 * 3,                            # m, n, w
               NBINS * NTW * 4 + NBINS * 8 + NTW * 8,    # M, w, G
               NTW * 8]
        alg_eval = alg[0] + alg[2]
    k = max(range(4), key=lambda i: kms[i])
    peak, peak_kind = _peaks()
    achieved = alg[k] / (kms[k] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": names[k], "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": _profile_traffic(names[k]),
                "peak_source": peak_kind,
                "kernel_ms": {n: kms[i] for i, n in enumerate(names)},
                "kernel_ms_back_to_back_warm_l2": kms_back_to_back[0],
                "fg_total_gbs": alg_eval / (ms / args.steps * 1e-3) / 1e9,
                "occupied_bin_plan": occupied,
                "autotuned_plan": {"path": path, "onepass_ms": H.onepass_ms,
                                   "onepass_variant": list(H.onepass_variant),
                                   "pass1_template_splits": tuned["plan"][0], "pass2_rows": tuned["plan"][1],
                                   "pass2_waves": tuned["plan"][2], "twopass_ms": tuned["ms"]}}

    # ---- end to end through the host-array C ABI (sfh_fg)
    comp = np.empty(NBINS)
    G = np.empty(NTW)
    h_r = r.copy()
    h_n = data.copy()
    for _ in range(3):
        sfhgpu.fg_(True, G, h_r, H, h_n, comp)
    ne2e = max(10, min(args.steps, 300))
    _barrier(world)
    e2e_s = 0.0
    for _ in range(ne2e):
        flush(tstream)  # outside the timed call
        tstream.synchronize()
        t0 = time.perf_counter()
        sfhgpu.fg_(True, G, h_r, H, h_n, comp)
        e2e_s += time.perf_counter() - t0
    e2e_s = _max_over_ranks(world, e2e_s)
    e2e = {"value": world * ne2e / e2e_s, "unit": UNIT, "h2d_bytes_per_step": (NTW + NBINS) * 8,
           "d2h_bytes_per_step": (NBINS + NTW + 1) * 8, "steps": ne2e}

    # ---- the rows beside the headline path (binary templates, bin_cmd, model_cmd)
    extras = None
    if not args.no_extras and rank == 0:
        extras = run_extras(ctx, w, cpu=not args.no_cpu)

    # ---- whole fits on the same templates (device BFGS driver vs a host scipy loop)
    fit = None
    if not args.no_fit:
        fit = run_fit(H, data)

    # ---- batched form (tensor cores): 4,096 vectors per call on the same templates
    batched = None
    if not args.no_batched:
        batched = run_batched(ctx, d_T, NBINS, NTW, r, data, M64, steps=5, warmup=2, B=args.batch)
        batched["speedup_vs_plain"] = batched["evals_per_s"] / value
        if occupied:
            batched["speedup_vs_plain_dense"] = batched["evals_per_s"] / occupied["dense_evals_per_s"]

    # ---- ragged galaxies: 256 uneven Hess grids, templates + fg! in one call each
    ragged = None
    if not args.no_ragged:
        ragged = run_ragged(ctx)

    # ---- learned template emulator (production grid), scored against exact templates
    emulator = None
    if not args.no_emulator:
        emulator = run_emulator(ctx, w, n_train=args.emu_train, steps=args.emu_steps)

    # ---- end-to-end hierarchical HMC (1,024 chains, MZR) on the same templates
    hmc = None
    if not args.no_hmc:
        hmc = run_hmc(ctx, d_T, w, nchains=args.hmc_chains, nwarmup=args.hmc_warmup,
                      ntraj=args.hmc_traj)
        hmc["speedup_vs_plain_evals"] = hmc["chain_gradient_evals_per_s"] / value
        if args.hmc_traj >= 100:  # not in short profiling runs
            hmc["matched_error"] = run_hmc_matched(ctx, d_T, w, nchains=args.hmc_chains)
        em = getattr(run_emulator, "last", None)
        if em is not None:
            # the same fit on emulated templates (exact where the trust map says so)
            la, mh = w.template_params
            th = np.stack([la, mh, np.full(la.size, w.dmod)], 1)
            d_em, used = em.templates(th, SyntheticGenerator(w.xedges, w.yedges, ctx=ctx))
            torch.cuda.synchronize()
            he = run_hmc(ctx, d_T, w, nchains=args.hmc_chains, nwarmup=args.hmc_warmup,
                         ntraj=args.hmc_traj, d_model=d_em)
            hmc["emulated_templates"] = {
                "emulated_fraction": float(np.mean(used)), "seconds": he["seconds"],
                "posterior_mean_alpha_MH0_sigma": he["posterior_mean_alpha_MH0_sigma"],
                "posterior_mean_abs_err": he["posterior_mean_abs_err"],
                "posterior_mean_R_rel_diff_vs_exact_templates_max": float(np.max(
                    np.abs(np.asarray(he["posterior_mean_R"]) / np.asarray(hmc["posterior_mean_R"])
                           - 1.0))),
            }
            del d_em

    # ---- CPU baseline (rank 0, N = 1 only): the oracle on the same inputs
    cpu = None
    plain_check = None
    if rank == 0 and world == 1 and not args.no_cpu:
        plain_check = oracle_checks(batched, ragged, M64, r, data, neglogl)
        plain_check["templates"] = template_checks(w, m_ini, mags, offs, lens, M32)
        v, thr, n, dt = cpu_fg_baseline(M64, r, data, budget_s=args.cpu_budget_s)
        tps, nt_done, tdt = cpu_template_baseline(w, budget_s=args.cpu_budget_s)
        cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{n} fg! evals in {dt:.1f} s (FP64 oracle, OpenMP {thr} threads)",
               "templates_per_s": tps,
               "templates_sample": f"{nt_done} partial_cmd_smooth templates in {tdt:.1f} s "
                                   f"(FP64 oracle, 1 thread)"}

    for leg in (batched, ragged):
        if leg:
            leg.pop("_check", None)  # unchecked (--no-cpu): no oracle run
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (compensated) + f64 logL",
            "data": "synthetic",
            "config": {"workload": WORKLOAD if NTW == NT else w.name, "nbins": NBINS,
                       "ntempl": NTW, "storage": "f32",
                       "l2": "flushed before every timed iteration (a write of twice the "
                             "L2 size, outside the timed intervals): the occupied-bin plan "
                             "streams 66 MB, which would fit in L2",
                       "parallelism": f"replicas x{world}"},
            "templates_per_s": templates_per_s, "template_build_ms": build_ms,
            "template_bin_updates_per_s": bin_updates / (build_ms / 1e3),
            "template_build_roofline": {
                "kernel": "k_stamps", "bound": "fp32 pipes (instruction issue)",
                "frac": _profile_value("fma_pipe_fraction k_stamps"),
                "issue_frac": _profile_value("issue_fraction k_stamps"),
                "unit": "FMA pipe share of its peak (ncu, profiles/k_stamps_production.md)"},
            "template_bin_updates_per_build": bin_updates,
            "negLogL": neglogl, "precision": plain_check, "gpu_launches": launches,
            "roofline": roofline,
            "batched": batched, "hmc": hmc, "ragged": ragged, "emulator": emulator, "fit": fit,
            "extras": extras,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    H.free()
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched tensor-core leg")
    ap.add_argument("--no-hmc", action="store_true", help="skip the batched HMC leg")
    ap.add_argument("--no-ragged", action="store_true", help="skip the ragged-galaxies leg")
    ap.add_argument("--fg-path", choices=("auto", "onepass", "twopass"), default="auto",
                    help="single-vector fg! path: the autotuner's choice (auto) or a fixed one "
                         "(for profiling runs, where profiler overhead can change the choice)")
    ap.add_argument("--no-emulator", action="store_true", help="skip the emulator leg")
    ap.add_argument("--no-fit", action="store_true", help="skip the whole-fit leg")
    ap.add_argument("--emu-train", type=int, default=150_000,
                    help="emulator training templates (smaller for a profiling case)")
    ap.add_argument("--emu-steps", type=int, default=60_000, help="emulator training steps")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the binary_hess / bin_cmd / model_cmd leg")
    ap.add_argument("--onepass-variant", default="",
                    help="pin the one-pass variant after autotuning: bins,ctas,schedule,boxes "
                         "(e.g. 32,1,phased,2)")
    ap.add_argument("--ntempl", type=int, default=NT,
                    help="templates (multiple of 30); fewer than 1200 only for profiling")
    ap.add_argument("--occupied", choices=("auto", "off", "on"), default="auto",
                    help="occupied-bin plan of the single-vector leg (off: the dense kernel "
                         "throughout, for profiling it)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the single-vector autotuner (profiling runs: fewer launches "
                         "before the timed ones; pin the variant with --onepass-variant)")
    ap.add_argument("--batch", type=int, default=4096,
                    help="coefficient vectors per batched call (4096: the batched workload)")
    ap.add_argument("--hmc-chains", type=int, default=1024)
    ap.add_argument("--hmc-warmup", type=int, default=500)
    ap.add_argument("--hmc-traj", type=int, default=1500,
                    help="sampling trajectories (fewer only for profiling runs)")
    ap.add_argument("--cpu-budget-s", type=float, default=10.0)
    ap.add_argument("--reference-budget-s", type=float, default=60.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
