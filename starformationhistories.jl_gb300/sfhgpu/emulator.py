"""Learned template emulator: MLP on a PCA basis, scored against and backed by exact templates.

No counterpart in the reference (a new component).  Parameters theta = (log age, [M/H],
distance modulus) are mapped by an MLP 3 -> 256 -> 256 -> 64 (GELU, FP32 master weights,
BF16-rounded matmul operands, trained with Adam by the library's own kernels,
``sfh_mlp_train``) to coefficients on a PCA basis of variance-stabilised templates
(y = sqrt(t)), centred and divided by one common scale so that the training loss is
proportional to the squared error in sqrt space (Poisson deviance ~ 4 sum (sqrt e -
sqrt t)^2).  Templates are rebuilt as t = max(0, offset + c V)^2.

The exact template (the GPU ``partial_cmd_smooth``) is both the arbiter and the fallback.
Score: Poisson deviance per star, D = 2 sum(e - t + t log(t/e)) / sum(t).  Routing: a
held-out validation set is scored by that deviance and the worst deviance seen in each cell
of a coarse grid over theta is kept (the trust map); a requested template is emulated
only when its cell was validated and its worst deviance is within tolerance, and is
built exactly otherwise.  ``templates(..., audit=True)`` instead builds every exact
template as well and falls back per template.

Everything heavy runs in libsfhgpu.so: template generation, the transform and
centring, the GEMMs of the randomized range finder (Halko, Martinsson & Tropp 2011,
Alg. 4.4 with power iterations), projection, training, inference, reconstruction and
the deviance score.  The host does only the small QR / SVD of the range finder (L x L and
n x L factors, L = K + 16) and bookkeeping.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, load
from .core import default_context

MODE_LINEAR, MODE_SQRT = 0, 1


def _torch():
    import torch
    return torch


@dataclass
class SyntheticGenerator:
    """Exact templates of the synthetic isochrone family at theta = (logAge, [M/H], dmod),
    built on the device by partial_cmd_smooth_batch.  Any callable with the same signature
    (theta (B x 3) numpy -> CUDA float32 tensor (B x nbins)) can drive the emulator."""
    xedges: np.ndarray
    yedges: np.ndarray
    n_iso: int = 400
    chunk: int = 2048
    ctx: object = None

    @property
    def nbins(self):
        return (self.xedges.size - 1) * (self.yedges.size - 1)

    def __call__(self, theta, out=None):
        from . import synthetic as S
        from .templates import partial_cmd_smooth_batch
        torch = _torch()
        ctx = self.ctx or default_context()
        dev = torch.device("cuda", ctx.device)
        theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
        B = theta.shape[0]
        if out is None:
            out = torch.empty((B, self.nbins), dtype=torch.float32, device=dev)
        for s in range(0, B, self.chunk):
            e = min(B, s + self.chunk)
            m, mags = S.isochrones(theta[s:e, 0], theta[s:e, 1], self.n_iso)
            nb = e - s
            offs = np.arange(nb, dtype=np.int64) * self.n_iso
            lens = np.full(nb, self.n_iso, dtype=np.int32)
            partial_cmd_smooth_batch(
                torch.as_tensor(m, device=dev), torch.as_tensor(mags, device=dev), offs, lens,
                1, (0, 1), S.error_models(), S.completeness_models(), S.imf(), theta[s:e, 2],
                1.0, (self.xedges, self.yedges), out=out[s:e], ctx=ctx)
        return out


def group_segments(group, max_rows=16):
    """(rows, seg) for sfh_emu_reconstruct_groups: row indices stably sorted by group, and
    one (group, start, count) triple per run of at most max_rows rows of one group."""
    group = np.asarray(group, dtype=np.int64).reshape(-1)
    rows = np.argsort(group, kind="stable").astype(np.int32)
    g = group[rows]
    n = g.size
    idx = np.arange(n)
    first = np.ones(n, dtype=bool)
    first[1:] = g[1:] != g[:-1]
    run0 = np.maximum.accumulate(np.where(first, idx, 0))   # start of each row's group run
    starts = np.nonzero(first | ((idx - run0) % max_rows == 0))[0]
    counts = np.diff(np.append(starts, n))
    return rows, np.stack([g[starts], starts, counts], 1).astype(np.int32).reshape(-1, 3)


@dataclass
class EmulatorReport:
    n_train: int
    n_val: int
    ncomp: int
    train_seconds: float
    generate_seconds: float
    pca_seconds: float
    final_loss: float
    val_deviance_quantiles: dict
    val_frac_within_tol: float
    trusted_cell_fraction: float
    loss_trace: np.ndarray = field(repr=False, default=None)


class TemplateEmulator:
    """MLP + PCA template emulator with exact-template arbiter and fallback."""

    def __init__(self, nbins, ncomp=64, hidden=(256, 256),
                 bounds=((6.6, 10.1), (-2.5, 0.3), (24.0, 30.0)), mode=MODE_SQRT,
                 tol=1e-3, cells=(12, 12, 12), basis_cells=None, trust_cells=None, ctx=None):
        """basis_cells=None: one global PCA basis and one MLP.  basis_cells=(na, nm, nd):
        one basis and one MLP per cell of that grid over theta (local form); the trust
        map then uses the same cells unless trust_cells gives a grid of its own (a finer
        one confines each failing validation template to a smaller cell; every cell needs
        validation templates of its own, so n_val grows with it)."""
        self.ctx = ctx or default_context()
        self.basis_cells = tuple(int(c) for c in basis_cells) if basis_cells else None
        if trust_cells:
            cells = trust_cells
        elif self.basis_cells:
            cells = self.basis_cells
        self.ngroups = int(np.prod(self.basis_cells)) if self.basis_cells else 1
        self.nbins = int(nbins)
        self.K = int(ncomp)
        self.shape = (3, int(hidden[0]), int(hidden[1]), self.K)
        self.bounds = np.asarray(bounds, dtype=np.float64)
        self.mode = int(mode)
        self.tol = float(tol)
        self.cells = tuple(int(c) for c in cells)
        self.trust = None       # worst validation deviance per cell (inf = unvalidated)
        self.params = None      # device FP32 parameter block
        self.basis = None       # device (K x nbins): sd-scaled PCA rows
        self.offset = None      # device (nbins): mean + mu_c V
        self.report = None
        L = load()
        n = C.c_int64()
        check(L.sfh_mlp_param_count(*self.shape, C.byref(n)), None, "mlp_param_count")
        self.nparams = n.value

    # ------------------------------------------------------------------ helpers
    @property
    def _dev(self):
        return _torch().device("cuda", self.ctx.device)

    def _sync_torch(self):
        _torch().cuda.current_stream(self._dev).synchronize()

    def _sync_ctx(self):
        check(load().sfh_ctx_synchronize(self.ctx.handle), self.ctx.handle, "synchronize")

    def standardize(self, theta):
        lo, hi = self.bounds[:, 0], self.bounds[:, 1]
        return (2.0 * (np.asarray(theta, dtype=np.float64) - lo) / (hi - lo) - 1.0)

    def group_of(self, theta):
        """Cell index of each theta in the basis grid (0 for the global form)."""
        theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
        if not self.basis_cells:
            return np.zeros(theta.shape[0], dtype=np.int64)
        lo, hi = self.bounds[:, 0], self.bounds[:, 1]
        n = np.asarray(self.basis_cells)
        idx = np.clip(((theta - lo) / (hi - lo) * n).astype(np.int64), 0, n - 1)
        return np.ravel_multi_index(idx.T, self.basis_cells)

    def local_inputs(self, theta):
        """MLP inputs: theta standardised to [-1, 1] over the whole box (global form) or
        over the theta's own basis cell (local form)."""
        theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
        if not self.basis_cells:
            return self.standardize(theta)
        lo, hi = self.bounds[:, 0], self.bounds[:, 1]
        n = np.asarray(self.basis_cells)
        w = (hi - lo) / n
        idx = np.clip(((theta - lo) / w).astype(np.int64), 0, n - 1)
        c_lo = lo + idx * w
        return 2.0 * (theta - c_lo) / w - 1.0

    def sample_theta(self, n, rng):
        lo, hi = self.bounds[:, 0], self.bounds[:, 1]
        return lo + (hi - lo) * rng.random((n, 3))

    def _gemm(self, A, B, Cout, M, N, K, ta, tb, accum=0, alpha=1.0, bf16=0):
        check(load().sfh_gemm_f32(self.ctx.handle, A.data_ptr(), B.data_ptr(), Cout.data_ptr(),
                                  M, N, K, ta, tb, accum, float(alpha), bf16),
              self.ctx.handle, "gemm_f32")

    def init_params(self, seed, ngroups=1):
        """Uniform(+-sqrt(6 / (fan_in + fan_out))) weights (Glorot), zero biases; one block
        per group, back to back."""
        rng = np.random.default_rng(seed)
        i, h1, h2, o = self.shape
        blocks = []
        for _ in range(ngroups):
            parts = []
            for fin, fout in ((i, h1), (h1, h2), (h2, o)):
                a = np.sqrt(6.0 / (fin + fout))
                parts += [rng.uniform(-a, a, fout * fin), np.zeros(fout)]
            blocks.append(np.concatenate(parts))
        p = np.concatenate(blocks).astype(np.float32)
        assert p.size == self.nparams * ngroups
        return p

    # ------------------------------------------------------------------ PCA
    def _pca(self, Y, n, rng, power_iters=3, oversample=16):
        """Top-K right singular vectors of the centred (n x nbins) device matrix Y by a
        randomized range finder with power iterations; returns (V (K x nbins) device,
        singular values)."""
        torch = _torch()
        L = self.K + oversample
        nb = self.nbins
        Om = torch.as_tensor(rng.standard_normal((nb, L)).astype(np.float32), device=self._dev)
        Z = torch.empty((n, L), dtype=torch.float32, device=self._dev)
        W = torch.empty((nb, L), dtype=torch.float32, device=self._dev)
        self._sync_torch()
        self._gemm(Y, Om, Z, n, L, nb, 0, 0)                       # Z = Y Om
        for _ in range(power_iters):
            self._sync_ctx()
            Q = np.linalg.qr(Z.cpu().numpy().astype(np.float64))[0].astype(np.float32)
            Z.copy_(torch.as_tensor(Q, device=self._dev))
            self._sync_torch()
            self._gemm(Y, Z, W, nb, L, n, 1, 0)                    # W = Y^T Q
            self._sync_ctx()
            Q = np.linalg.qr(W.cpu().numpy().astype(np.float64))[0].astype(np.float32)
            W.copy_(torch.as_tensor(Q, device=self._dev))
            self._sync_torch()
            self._gemm(Y, W, Z, n, L, nb, 0, 0)                    # Z = Y Q
        self._sync_ctx()
        Q = np.linalg.qr(Z.cpu().numpy().astype(np.float64))[0].astype(np.float32)
        Z.copy_(torch.as_tensor(Q, device=self._dev))
        Bm = torch.empty((L, nb), dtype=torch.float32, device=self._dev)
        self._sync_torch()
        self._gemm(Z, Y, Bm, L, nb, n, 1, 0)                       # B = Q^T Y
        self._sync_ctx()
        Bh = Bm.cpu().numpy().astype(np.float64)
        # SVD of the small L x nb factor through its L x L Gram matrix
        ev, U = np.linalg.eigh(Bh @ Bh.T)
        order = np.argsort(ev)[::-1][: self.K]
        sv = np.sqrt(np.maximum(ev[order], 0.0))
        V = (U[:, order].T @ Bh) / np.where(sv > 0, sv, 1.0)[:, None]
        return torch.as_tensor(V.astype(np.float32), device=self._dev), sv

    # ------------------------------------------------------------------ training
    def fit(self, generator, n_train=100_000, n_val=4096, steps=20_000, batch=1024, lr=1e-3,
            lr_final=1e-5, seed=20261203, segments=20, power_iters=3, batch_per_cell=32):
        """Generate n_train exact templates on the device, build the PCA basis (global, or
        one per basis cell), train the MLP(s) (Adam, cosine-decayed from lr to lr_final over
        `steps` in `segments` calls; global: `batch` rows per step, local: `batch_per_cell`
        rows per cell per step), then score n_val fresh templates by deviance to build
        the trust map."""
        torch = _torch()
        L = load()
        rng = np.random.default_rng(seed)
        theta = self.sample_theta(n_train, rng)
        grp = self.group_of(theta)
        order = np.argsort(grp, kind="stable")
        theta, grp = theta[order], grp[order]
        off = np.searchsorted(grp, np.arange(self.ngroups + 1)).astype(np.int64)
        if np.any(np.diff(off) < 2):
            raise ValueError("too few training templates: every basis cell needs at least two")
        t0 = time.perf_counter()
        Y = generator(theta)
        torch.cuda.synchronize(self._dev)
        t_gen = time.perf_counter() - t0

        t0 = time.perf_counter()
        if self.basis_cells:
            T = self._local_basis(Y, off)
        else:
            T = self._global_basis(Y, n_train, rng, power_iters)
        del Y
        X = torch.as_tensor(self.local_inputs(theta).astype(np.float32), device=self._dev)
        torch.cuda.synchronize(self._dev)
        t_pca = time.perf_counter() - t0

        t0 = time.perf_counter()
        self.params = torch.as_tensor(self.init_params(seed, self.ngroups), device=self._dev)
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        trace = torch.empty(max(steps, 1), dtype=torch.float32, device=self._dev)
        self._sync_torch()
        done = 0
        per = max(1, -(-steps // max(1, segments)))
        while done < steps:
            k = min(per, steps - done)
            frac = (done + 0.5 * k) / steps
            lr_k = lr_final + 0.5 * (lr - lr_final) * (1.0 + np.cos(np.pi * frac))
            tp = trace.data_ptr() + 4 * done
            if self.basis_cells:
                check(L.sfh_mlp_train_grouped(
                    self.ctx.handle, *self.shape, self.ngroups, self.params.data_ptr(),
                    m.data_ptr(), v.data_ptr(), done, X.data_ptr(), T.data_ptr(),
                    off.ctypes.data, int(batch_per_cell), k, float(lr_k), seed, tp),
                    self.ctx.handle, "mlp_train_grouped")
            else:
                check(L.sfh_mlp_train(self.ctx.handle, *self.shape, self.params.data_ptr(),
                                      m.data_ptr(), v.data_ptr(), done, X.data_ptr(),
                                      T.data_ptr(), n_train, batch, k, float(lr_k), seed, tp),
                      self.ctx.handle, "mlp_train")
            done += k
        t_train = time.perf_counter() - t0
        tr = trace[:steps].cpu().numpy()

        # score on a held-out set -> trust map
        th_val = self.sample_theta(n_val, rng)
        dev = self.deviance(th_val, generator(th_val))
        self._build_trust(th_val, dev)
        q = np.quantile(dev, [0.1, 0.5, 0.9, 0.99])
        self.report = EmulatorReport(
            n_train=n_train, n_val=n_val, ncomp=self.K, train_seconds=t_train,
            generate_seconds=t_gen, pca_seconds=t_pca,
            final_loss=float(np.mean(tr[-max(1, steps // 100):])) if steps else float("nan"),
            val_deviance_quantiles=dict(zip(("q10", "q50", "q90", "q99"), map(float, q))),
            val_frac_within_tol=float(np.mean(dev <= self.tol)),
            trusted_cell_fraction=float(np.mean(self.trust <= self.tol)), loss_trace=tr)
        return self.report

    def _global_basis(self, Y, n, rng, power_iters):
        """One basis for all templates (randomized range finder); returns the MLP targets
        and sets basis / offset with the coefficient scaling folded in."""
        torch = _torch()
        L = load()
        mean = torch.empty(self.nbins, dtype=torch.float32, device=self._dev)
        check(L.sfh_emu_prepare(self.ctx.handle, Y.data_ptr(), n, self.nbins, self.mode,
                                mean.data_ptr()), self.ctx.handle, "emu_prepare")
        V, sv = self._pca(Y, n, rng, power_iters=power_iters)
        A = torch.empty((n, self.K), dtype=torch.float32, device=self._dev)
        self._sync_torch()
        self._gemm(Y, V, A, n, self.K, self.nbins, 0, 1)     # A = Y V^T
        self._sync_ctx()
        Ah = A.cpu().numpy().astype(np.float64)
        # one common scale for all components: the MSE is then proportional to the
        # squared error in sqrt-template space, which is what the deviance score sees
        cmu = Ah.mean(0)
        s = float(np.sqrt(np.mean(Ah.var(0)))) or 1.0
        Vh = V.cpu().numpy().astype(np.float64)
        self.basis = torch.as_tensor((s * Vh).astype(np.float32), device=self._dev)
        self.offset = torch.as_tensor(
            (mean.cpu().numpy().astype(np.float64) + cmu @ Vh).astype(np.float32),
            device=self._dev)
        self.singular_values = sv
        return torch.as_tensor(((Ah - cmu) / s).astype(np.float32), device=self._dev)

    def _local_basis(self, Y, off):
        """One basis per cell from the cell's Gram matrix (n_c x n_c on the device, its
        eigenproblem on the host): V_c = diag(1/sqrt(l)) U^T Y_c and training coefficients
        U sqrt(l).  Sets basis (G x K x nbins) and offset (G x nbins)."""
        torch = _torch()
        L = load()
        G, K, nb = self.ngroups, self.K, self.nbins
        self.basis = torch.zeros((G, K, nb), dtype=torch.float32, device=self._dev)
        self.offset = torch.empty((G, nb), dtype=torch.float32, device=self._dev)
        T = np.zeros((int(off[-1]), K), dtype=np.float32)
        sv = []
        for g in range(G):
            a, b = int(off[g]), int(off[g + 1])
            n = b - a
            Yg = Y[a:b]
            mean = self.offset[g]
            self._sync_torch()
            check(L.sfh_emu_prepare(self.ctx.handle, Yg.data_ptr(), n, nb, self.mode,
                                    mean.data_ptr()), self.ctx.handle, "emu_prepare")
            Gm = torch.empty((n, n), dtype=torch.float32, device=self._dev)
            self._gemm(Yg, Yg, Gm, n, n, nb, 0, 1)               # Y_c Y_c^T
            self._sync_ctx()
            ev, U = np.linalg.eigh(Gm.cpu().numpy().astype(np.float64))
            ev, U = ev[::-1], U[:, ::-1]
            k = int(min(K, n - 1, np.sum(ev > ev[0] * 1e-12)))
            lam = ev[:k]
            Us = U[:, :k] / np.sqrt(lam)[None, :]
            Ud = torch.as_tensor(np.ascontiguousarray(Us, dtype=np.float32), device=self._dev)
            Vg = self.basis[g, :k]
            self._sync_torch()
            self._gemm(Ud, Yg, Vg, k, nb, n, 1, 0)                # diag(1/sqrt l) U^T Y_c
            A = U[:, :k] * np.sqrt(lam)[None, :]                  # = Y_c V_c^T
            s = float(np.sqrt(np.mean(A.var(0)))) or 1.0
            cmu = A.mean(0)
            T[a:b, :k] = (A - cmu) / s
            self._sync_ctx()
            Vh = Vg.cpu().numpy().astype(np.float64)
            mean_h = mean.cpu().numpy().astype(np.float64)
            self.offset[g] = torch.as_tensor((mean_h + cmu @ Vh).astype(np.float32),
                                             device=self._dev)
            Vg.mul_(s)
            sv.append(np.sqrt(lam))
        self.singular_values = sv
        torch.cuda.synchronize(self._dev)
        return torch.as_tensor(T, device=self._dev)

    # ------------------------------------------------------------------ inference
    def coefficients(self, theta):
        """Scaled PCA coefficients predicted by the MLP(s) (device, B x K)."""
        torch = _torch()
        theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
        if theta.shape[0] == 0:
            return torch.empty((0, self.K), dtype=torch.float32, device=self._dev)
        X = torch.as_tensor(self.local_inputs(theta).astype(np.float32), device=self._dev)
        B = X.shape[0]
        Yc = torch.empty((B, self.K), dtype=torch.float32, device=self._dev)
        grp = torch.as_tensor(self.group_of(theta).astype(np.int32), device=self._dev)
        self._sync_torch()
        if self.basis_cells:
            check(load().sfh_mlp_forward_rows(self.ctx.handle, *self.shape,
                                              self.params.data_ptr(), self.ngroups,
                                              X.data_ptr(), grp.data_ptr(), B, Yc.data_ptr()),
                  self.ctx.handle, "mlp_forward_rows")
            self._sync_ctx()
        else:
            check(load().sfh_mlp_forward(self.ctx.handle, *self.shape, self.params.data_ptr(),
                                         X.data_ptr(), B, Yc.data_ptr()), self.ctx.handle,
                  "mlp_forward")
        return Yc

    def predict(self, theta, out=None):
        """Emulated templates (device float32, B x nbins)."""
        torch = _torch()
        theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
        coef = self.coefficients(theta)
        B = coef.shape[0]
        if out is None:
            out = torch.empty((B, self.nbins), dtype=torch.float32, device=self._dev)
        if B == 0:
            return out
        L = load()
        if self.basis_cells:
            # rows sorted by cell, in segments of at most 16: each cell's basis is read once
            # per segment rather than once per row
            rows, seg = group_segments(self.group_of(theta))
            d_rows = torch.as_tensor(rows, device=self._dev)
            d_seg = torch.as_tensor(seg, device=self._dev)
            self._sync_torch()
            for s0 in range(0, seg.shape[0], 65535):
                e = min(seg.shape[0], s0 + 65535)
                check(L.sfh_emu_reconstruct_groups(
                    self.ctx.handle, coef.data_ptr(), d_rows.data_ptr(), d_seg[s0:e].data_ptr(),
                    e - s0, self.ngroups, self.basis.data_ptr(), self.offset.data_ptr(), self.K,
                    self.nbins, B, self.mode, out.data_ptr()), self.ctx.handle,
                    "emu_reconstruct_groups")
        else:
            check(L.sfh_emu_reconstruct(self.ctx.handle, coef.data_ptr(), self.basis.data_ptr(),
                                        self.offset.data_ptr(), self.K, self.nbins, B, self.mode,
                                        out.data_ptr()), self.ctx.handle, "emu_reconstruct")
        self._sync_ctx()
        return out

    def score(self, exact, emul):
        """Poisson deviance per star of each emulated row against the exact row (numpy)."""
        torch = _torch()
        B = exact.shape[0]
        d = torch.empty(B, dtype=torch.float64, device=self._dev)
        self._sync_torch()
        check(load().sfh_poisson_deviance(self.ctx.handle, exact.data_ptr(), emul.data_ptr(),
                                          self.nbins, B, d.data_ptr()), self.ctx.handle,
              "poisson_deviance")
        self._sync_ctx()
        return d.cpu().numpy()

    def deviance(self, theta, exact):
        return self.score(exact, self.predict(theta))

    # ------------------------------------------------------------------ routing
    def _cell(self, theta):
        lo, hi = self.bounds[:, 0], self.bounds[:, 1]
        u = (np.asarray(theta, dtype=np.float64).reshape(-1, 3) - lo) / (hi - lo)
        idx = np.clip((u * np.asarray(self.cells)).astype(np.int64), 0,
                      np.asarray(self.cells) - 1)
        inside = np.all((u >= 0) & (u <= 1), axis=1)
        return np.ravel_multi_index(idx.T, self.cells), inside

    def _build_trust(self, theta, dev):
        trust = np.full(int(np.prod(self.cells)), np.inf)
        cell, inside = self._cell(theta)
        for c, d in zip(cell[inside], dev[inside]):
            trust[c] = d if not np.isfinite(trust[c]) else max(trust[c], d)
        self.trust = trust

    def trusted(self, theta):
        cell, inside = self._cell(theta)
        return inside & (self.trust[cell] <= self.tol)

    def templates(self, theta, generator, audit=False):
        """Templates for theta (B x 3): emulated where trusted, exact elsewhere.  With
        audit=True every exact template is built too and each emulated one that the deviance score
        rejects is replaced.  Returns (templates (device B x nbins), emulated mask)."""
        theta = np.asarray(theta, dtype=np.float64).reshape(-1, 3)
        out = self.predict(theta)
        if audit:
            exact = generator(theta)
            dev = self.score(exact, out)
            use = dev <= self.tol
        else:
            use = self.trusted(theta)
        bad = np.nonzero(~use)[0]
        if bad.size:
            torch = _torch()
            if audit:
                idx = torch.as_tensor(bad, device=self._dev)
                out[idx] = exact[idx]
            else:
                out[torch.as_tensor(bad, device=self._dev)] = generator(theta[bad])
        return out, use
