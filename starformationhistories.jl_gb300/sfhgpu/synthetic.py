"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No observational dataset is involved: isochrones are smooth analytic functions of
initial mass, so every number here is reproducible from the seed.

Isochrone model (three filters B, V, R; index 0, 1, 2):
  x = log10(m), t = logAge - 6.6, turn-off log-mass xTO = log10(1.45) - 0.07 t,
  g(x) = (1 + tanh((x - xTO) / 0.02)) / 2          (0 on the main sequence, 1 on giants)
  V = 4.8 - 7.5 x + 0.3 t - 6 g(x)                  (monotone in mass; +0.3 mag per dex of age)
  B - V = 0.65 - 1.1 x + 0.2 [M/H] + 0.9 g(x) (1 - 0.3 t / 3.5)
  B = V + (B - V),  R = V - 0.55 (B - V)
  m_ini: 400 points log-spaced on [0.1, 1.5] Msun.
Photometric error sigma(m) = 0.01 + 0.3 exp((m - 28)/1.2) = exp_photerr(m, e, 1/1.2,
28 - 1.2 ln 0.3, 0.01); completeness Martin2016(m, 1, 28, 0.3); Kroupa2001(0.08, 100) IMF;
distance modulus 25.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .templates import Kroupa2001, compl_model, err_model

SEED = 20261203
DMOD = 25.0


def isochrone(logAge: float, MH: float, n: int = 400):
    """(m_ini[n], mags[3, n]) for filters (B, V, R), absolute magnitudes."""
    m = np.logspace(np.log10(0.1), np.log10(1.5), n)
    x = np.log10(m)
    t = logAge - 6.6
    xto = np.log10(1.45) - 0.07 * t
    g = 0.5 * (1.0 + np.tanh((x - xto) / 0.02))
    V = 4.8 - 7.5 * x + 0.3 * t - 6.0 * g
    BV = 0.65 - 1.1 * x + 0.2 * MH + 0.9 * g * (1.0 - 0.3 * t / 3.5)
    return m, np.stack([V + BV, V, V - 0.55 * BV])


def isochrones(logAge, MH, n: int = 400):
    """Vectorised isochrone() over B templates: (m_ini[B*n], mags[3, B*n]) with template
    b's points at [b*n, (b+1)*n)."""
    logAge = np.asarray(logAge, dtype=np.float64).reshape(-1, 1)
    MH = np.asarray(MH, dtype=np.float64).reshape(-1, 1)
    m = np.logspace(np.log10(0.1), np.log10(1.5), n)[None, :]
    x = np.log10(m)
    t = logAge - 6.6
    xto = np.log10(1.45) - 0.07 * t
    g = 0.5 * (1.0 + np.tanh((x - xto) / 0.02))
    V = 4.8 - 7.5 * x + 0.3 * t - 6.0 * g
    BV = 0.65 - 1.1 * x + 0.2 * MH + 0.9 * g * (1.0 - 0.3 * t / 3.5)
    B = logAge.shape[0]
    mags = np.stack([(V + BV).ravel(), np.broadcast_to(V, (B, n)).ravel(),
                     (V - 0.55 * BV).ravel()])
    return np.broadcast_to(m, (B, n)).ravel().copy(), mags


@dataclass
class Workload:
    name: str
    logAges: np.ndarray
    MHs: np.ndarray
    xedges: np.ndarray
    yedges: np.ndarray
    y_index: int = 1              # V on the y axis
    color_indices: tuple = (0, 1)  # B - V on the x axis (covariant kernel, cov_mult = +1)
    n_iso: int = 400
    n_stars: float = 1e4
    dmod: float = DMOD
    normalize_value: float = 1.0
    seed: int = SEED
    extra: dict = field(default_factory=dict)

    @property
    def grid(self):
        return (self.xedges.size - 1, self.yedges.size - 1)

    @property
    def nbins(self):
        nx, ny = self.grid
        return nx * ny

    @property
    def template_params(self):
        """(logAge, [M/H]) per template: logAge outer, [M/H] inner."""
        la = np.repeat(self.logAges, self.MHs.size)
        mh = np.tile(self.MHs, self.logAges.size)
        return la, mh

    @property
    def ntempl(self):
        return self.logAges.size * self.MHs.size


def _edges(nx, ny):
    return np.linspace(-0.6, 2.4, nx + 1), np.linspace(19.0, 30.0, ny + 1)


def config1(**kw) -> Workload:
    """Plain method, FP64, CPU-runnable: 10 ages x 5 [M/H] = 50 templates on 75 x 100 bins,
    1e4 stars."""
    xe, ye = _edges(75, 100)
    return Workload("config1: 50 templates, 75x100 Hess grid, 1e4 stars",
                    np.linspace(6.6, 10.1, 10), np.linspace(-2.0, 0.0, 5), xe, ye, n_stars=1e4,
                    **kw)


def config2(**kw) -> Workload:
    """Production size: 40 ages x 30 [M/H] = 1,200 templates on 200 x 300 bins, 1e6 stars."""
    xe, ye = _edges(200, 300)
    return Workload("config2: 1200 templates, 200x300 Hess grid, 1e6 stars",
                    np.linspace(6.6, 10.1, 40), np.linspace(-2.5, 0.3, 30), xe, ye, n_stars=1e6,
                    **kw)


def small(nages=3, nmh=2, nx=40, ny=50, n_iso=120, **kw) -> Workload:
    """A small case with the same generators, for fast parity tests."""
    xe, ye = _edges(nx, ny)
    return Workload(f"small: {nages * nmh} templates, {nx}x{ny}", np.linspace(6.6, 10.1, nages),
                    np.linspace(-2.0, 0.0, nmh), xe, ye, n_iso=n_iso, **kw)


def error_models(nf=3):
    a, b, c, d = np.e, 1.0 / 1.2, 28.0 - 1.2 * np.log(0.3), 0.01
    return [err_model(a, b, c, d, np.inf) for _ in range(nf)]


def error_funcs(nf=3):
    a, b, c, d = np.e, 1.0 / 1.2, 28.0 - 1.2 * np.log(0.3), 0.01
    return [(lambda m, a=a, b=b, c=c, d=d: a ** (b * (np.asarray(m) - c)) + d)
            for _ in range(nf)]


def completeness_models(nf=3):
    return [compl_model(1.0, 28.0, 0.3) for _ in range(nf)]


def completeness_funcs(nf=3):
    return [(lambda m: 1.0 / (1.0 + np.exp((np.asarray(m) - 28.0) / 0.3))) for _ in range(nf)]


def imf():
    return Kroupa2001(0.08, 100.0)


def isochrone_batch(w: Workload):
    """Concatenated isochrones of all templates: (m_ini[total], mags[3, total], off, len)."""
    la, mh = w.template_params
    ms, mg = [], []
    for a, z in zip(la, mh):
        m, mags = isochrone(a, z, w.n_iso)
        ms.append(m)
        mg.append(mags)
    m_ini = np.concatenate(ms)
    mags = np.concatenate(mg, axis=1)
    lens = np.full(w.ntempl, w.n_iso, dtype=np.int32)
    offs = np.arange(w.ntempl, dtype=np.int64) * w.n_iso
    return m_ini, mags, offs, lens


def coefficients(nt: int, seed: int = SEED, B: int | None = None):
    """exp(N(0,1)) coefficient vectors (one vector, or B x nt)."""
    rng = np.random.default_rng(seed)
    shape = (nt,) if B is None else (B, nt)
    return np.exp(rng.standard_normal(shape))


def observed(models_f64: np.ndarray, n_stars: float, seed: int = SEED):
    """(coeffs, data): exp(N(0,1)) coefficients scaled so the composite holds n_stars
    stars, and a Poisson draw of that composite."""
    nt = models_f64.shape[1]
    r = coefficients(nt, seed)
    m = models_f64 @ r
    r = r * (n_stars / m.sum())
    m = models_f64 @ r
    rng = np.random.default_rng(seed + 1)
    return r, rng.poisson(m).astype(np.float64)


@dataclass
class Galaxy:
    """One galaxy of the ragged workload: its own Hess grid, isochrone length, ages,
    metallicities and distance modulus."""
    xedges: np.ndarray
    yedges: np.ndarray
    n_iso: int
    logAges: np.ndarray
    MHs: np.ndarray
    dmod: float

    @property
    def grid(self):
        return (self.xedges.size - 1, self.yedges.size - 1)

    @property
    def nbins(self):
        nx, ny = self.grid
        return nx * ny

    @property
    def ntempl(self):
        return self.logAges.size * self.MHs.size


def ragged(ngal=256, nages=4, nmh=3, nxy=(50, 300), niso=(100, 2000), seed=SEED):
    """Independent galaxies with uneven Hess grids (nx, ny uniform on nxy per axis, over
    the same colour / magnitude window) and uneven isochrone lengths (uniform on niso);
    ages uniform on [6.6, 10.1], [M/H] on [-2.5, 0.3], distance modulus on [24.5, 26.5]."""
    rng = np.random.default_rng(seed + 7)
    out = []
    for _ in range(ngal):
        nx, ny = (int(v) for v in rng.integers(nxy[0], nxy[1] + 1, 2))
        xe, ye = _edges(nx, ny)
        out.append(Galaxy(xe, ye, int(rng.integers(niso[0], niso[1] + 1)),
                          np.sort(rng.uniform(6.6, 10.1, nages)), rng.uniform(-2.5, 0.3, nmh),
                          float(rng.uniform(24.5, 26.5))))
    return out


def ragged_isochrones(galaxies):
    """Concatenated isochrones of every template of every galaxy (galaxy-major, then
    log age, then [M/H]): (m_ini, mags[3, total], iso_off, iso_len, dmod per template,
    (xedges, yedges) per template)."""
    ms, mg, lens, dm, edges = [], [], [], [], []
    for g in galaxies:
        la = np.repeat(g.logAges, g.MHs.size)
        mh = np.tile(g.MHs, g.logAges.size)
        m, mags = isochrones(la, mh, g.n_iso)
        ms.append(m)
        mg.append(mags)
        lens += [g.n_iso] * la.size
        dm += [g.dmod] * la.size
        edges += [(g.xedges, g.yedges)] * la.size
    lens = np.asarray(lens, dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    return np.concatenate(ms), np.concatenate(mg, axis=1), offs, lens, np.asarray(dm), edges
