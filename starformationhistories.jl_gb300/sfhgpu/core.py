"""Contexts and template-matrix handles (sfh_ctx / sfh_models of include/sfhgpu.h)."""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _lib
from ._lib import SFH_BF16X2, SFH_F32, SFH_F64, check, load, ptr

_STORAGE = {"f64": SFH_F64, "f32": SFH_F32, "bf16x2": SFH_BF16X2,
            SFH_F64: SFH_F64, SFH_F32: SFH_F32, SFH_BF16X2: SFH_BF16X2}


class Context:
    """One CUDA stream plus scratch on one device (sfh_ctx_create).  Use one per thread."""

    def __init__(self, device: int = 0):
        L = load()
        h = C.c_void_p()
        check(L.sfh_ctx_create(int(device), C.byref(h)), None, "sfh_ctx_create")
        self._h = h
        self.device = int(device)

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("context destroyed")
        return self._h

    def synchronize(self):
        check(load().sfh_ctx_synchronize(self.handle), self.handle, "synchronize")

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(load().sfh_ctx_stream(self.handle, C.byref(s)), self.handle)
        return int(s.value or 0)

    @property
    def launches(self) -> int:
        n = C.c_int64()
        check(load().sfh_ctx_launch_count(self.handle, C.byref(n)), self.handle)
        return int(n.value)

    def set_wait_budget(self, cycles: int = 0):
        """Budget of each bounded device wait of the single-vector pipeline, in SM cycles
        (0: the default, about 2 s)."""
        check(load().sfh_ctx_set_wait_budget(self.handle, int(cycles)), self.handle)

    def inject_fault(self, what: int):
        """One-shot failure injection for tests of the error paths (SFH_INJECT_*)."""
        check(load().sfh_ctx_inject_fault(self.handle, int(what)), self.handle)

    def set_overlap(self, on: bool = True):
        """Overlap back-to-back single-vector fg! launches (sfh_ctx_set_overlap)."""
        check(load().sfh_ctx_set_overlap(self.handle, 1 if on else 0), self.handle)

    @property
    def host_access(self) -> int:
        """How sfh_fg reaches host arrays: SFH_HOST_ACCESS_STAGED (mapped pinned staging)
        or SFH_HOST_ACCESS_DIRECT (the kernels use the caller's arrays)."""
        m = C.c_int()
        check(load().sfh_ctx_host_access(self.handle, C.byref(m)), self.handle)
        return int(m.value)

    @host_access.setter
    def host_access(self, mode: int):
        check(load().sfh_ctx_set_host_access(self.handle, int(mode)), self.handle)

    def torch_stream(self):
        import torch
        return torch.cuda.ExternalStream(self.stream, device=torch.device("cuda", self.device))

    def close(self):
        if getattr(self, "_h", None) is not None:
            load().sfh_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


_tls = threading.local()


def default_context() -> Context:
    ctx = getattr(_tls, "ctx", None)
    if ctx is None:
        ctx = Context(0)
        _tls.ctx = ctx
    return ctx


class Models:
    """Device-resident template matrix in the flattened layout (nbins, ntemplates),
    one template per column (stack_models, src/fitting/utilities.jl:12-13)."""

    def __init__(self, M=None, storage="f32", ctx: Context | None = None, _handle=None,
                 _shape=None):
        self.ctx = ctx or default_context()
        L = load()
        self.storage = _STORAGE[storage]
        if _handle is not None:
            self._h = _handle
            self.nbins, self.nt = _shape
            return
        A = np.asarray(M)
        if A.ndim != 2:
            raise ValueError("models must be a (nbins, ntemplates) matrix")
        src = SFH_F32 if A.dtype == np.float32 else SFH_F64
        A = np.asfortranarray(A, dtype=np.float32 if src == SFH_F32 else np.float64)
        self.nbins, self.nt = A.shape
        h = C.c_void_p()
        check(L.sfh_models_upload(self.ctx.handle, A.ctypes.data, src, self.nbins, self.nt,
                                  self.storage, C.byref(h)), self.ctx.handle, "sfh_models_upload")
        self._h = h

    @classmethod
    def from_device(cls, dev_ptr: int, nbins: int, nt: int, storage="f32",
                    ctx: Context | None = None):
        """Wrap device FP32 (nbins, nt) column-major templates (copied)."""
        ctx = ctx or default_context()
        h = C.c_void_p()
        st = _STORAGE[storage]
        check(load().sfh_models_from_device(ctx.handle, int(dev_ptr), int(nbins), int(nt), st,
                                            C.byref(h)), ctx.handle, "sfh_models_from_device")
        return cls(ctx=ctx, storage=st, _handle=h, _shape=(int(nbins), int(nt)))

    @property
    def handle(self):
        return self._h

    @property
    def shape(self):
        return (self.nbins, self.nt)

    def combine(self, groups, weights, storage="f32"):
        """A new matrix whose column g is sum(weights[g][q] * self[:, groups[g][q]]): one
        pass over this matrix on the device (sfh_models_combine)."""
        off = np.zeros(len(groups) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(gr) for gr in groups])
        cols = np.ascontiguousarray(np.concatenate([np.asarray(gr) for gr in groups]),
                                    dtype=np.int32)
        w = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.float64)
                                                 for x in weights]))
        st = {"f32": SFH_F32, "bf16x2": SFH_BF16X2}[storage]
        h = C.c_void_p()
        check(load().sfh_models_combine(self.ctx.handle, self._h, len(groups), off.ctypes.data,
                                        cols.ctypes.data, w.ctypes.data, st, C.byref(h)),
              self.ctx.handle, "models_combine")
        return Models(ctx=self.ctx, storage=st, _handle=h, _shape=(self.nbins, len(groups)))

    PATHS = {"auto": 0, "onepass": 1, "twopass": 2}

    def set_path(self, path):
        """Single-vector fg! path for calls with G: "onepass" (one read of the matrix;
        FP32 storage, nt <= 1536; keeps a blocked copy of the templates), "twopass" or
        "auto" (sfh_models_set_path)."""
        check(load().sfh_models_set_path(self.ctx.handle, self._h, self.PATHS[path]),
              self.ctx.handle, "models_set_path")

    def set_onepass_tile(self, bins):
        """Bins per tile of the one-pass kernel: 16 or 32 (sfh_models_set_onepass_tile)."""
        check(load().sfh_models_set_onepass_tile(self.ctx.handle, self._h, int(bins)),
              self.ctx.handle, "models_set_onepass_tile")

    def set_onepass_ctas(self, per_sm):
        """CTAs per SM of the one-pass kernel: 1 or 2 (sfh_models_set_onepass_ctas)."""
        check(load().sfh_models_set_onepass_ctas(self.ctx.handle, self._h, int(per_sm)),
              self.ctx.handle, "models_set_onepass_ctas")

    def set_onepass_schedule(self, schedule):
        """Schedule of the one-pass kernel: "phased" or "skewed"
        (sfh_models_set_onepass_schedule)."""
        _s = {"phased": 0, "skewed": 1}[schedule]
        check(load().sfh_models_set_onepass_schedule(self.ctx.handle, self._h, _s),
              self.ctx.handle, "models_set_onepass_schedule")

    def set_onepass_run(self, boxes):
        """Boxes per bulk copy of the one-pass kernel: 1, 2, 4 or 0 for the default
        (sfh_models_set_onepass_run)."""
        check(load().sfh_models_set_onepass_run(self.ctx.handle, self._h, int(boxes)),
              self.ctx.handle, "models_set_onepass_run")

    OCC = {"off": 0, "auto": 1, "on": 2}

    def set_occupied(self, mode):
        """Occupied-bin restriction of fg! with G (sfh_models_set_occupied): "off" (the
        dense kernel), "auto" (default: a plan per observed diagram when at most 60 % of
        its bins hold counts) or "on"."""
        check(load().sfh_models_set_occupied(self.ctx.handle, self._h, self.OCC[mode]),
              self.ctx.handle, "models_set_occupied")

    def occupied_info(self, data_ptr=None):
        """(occupied bins or -1, restricted kernel in use, last plan build ms) of the plan
        for the device data pointer (None: the host-array calls' slot)."""
        n, sp, ms = C.c_int64(), C.c_int(), C.c_double()
        key = data_ptr if data_ptr is not None else self._h
        check(load().sfh_models_occupied_info(self.ctx.handle, self._h, key, C.byref(n),
                                              C.byref(sp), C.byref(ms)),
              self.ctx.handle, "models_occupied_info")
        return int(n.value), bool(sp.value), float(ms.value)

    @property
    def onepass_variant(self):
        """(bins per tile, CTAs per SM, schedule, boxes per bulk copy) of the one-pass
        launches."""
        b, c, k, r = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(load().sfh_models_onepass_variant(self.ctx.handle, self._h, C.byref(b), C.byref(c),
                                                C.byref(k), C.byref(r)), self.ctx.handle,
              "models_onepass_variant")
        return b.value, c.value, ("skewed" if k.value else "phased"), r.value

    @property
    def path(self):
        """The path fg! calls with G take on this handle now: "onepass" or "twopass"."""
        p = C.c_int()
        check(load().sfh_models_path(self.ctx.handle, self._h, C.byref(p), None), self.ctx.handle,
              "models_path")
        return {1: "onepass", 2: "twopass"}[p.value]

    @property
    def onepass_ms(self):
        """One-pass fg! time measured by autotune (0.0 if not measured)."""
        ms = C.c_double()
        check(load().sfh_models_path(self.ctx.handle, self._h, None, C.byref(ms)), self.ctx.handle,
              "models_path")
        return ms.value

    def autotune(self, coeffs, data, iters=10, eps=None):
        """Pick the fastest single-vector fg! launch plan for this matrix by timing the
        candidates on the device (sfh_models_autotune).  Returns
        {"plan": (pass-1 template splits, pass-2 rows, pass-2 waves), "ms": (pass 1, pass 2)}."""
        import torch
        dev = torch.device("cuda", self.ctx.device)
        r = torch.as_tensor(np.asarray(coeffs, dtype=np.float64), device=dev).contiguous()
        n = torch.as_tensor(np.asarray(data, dtype=np.float64).reshape(-1), device=dev).contiguous()
        plan = (C.c_int * 3)()
        ms = (C.c_double * 2)()
        eps = float(np.finfo(np.float64).eps) if eps is None else float(eps)
        torch.cuda.current_stream(dev).synchronize()
        check(load().sfh_models_autotune(self.ctx.handle, self._h, r.data_ptr(), n.data_ptr(), eps,
                                         int(iters), plan, ms), self.ctx.handle, "autotune")
        return {"plan": tuple(plan), "ms": tuple(ms)}

    def free(self):
        if getattr(self, "_h", None) is not None:
            load().sfh_models_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:  # noqa: BLE001
            pass


def as_models(models, dtype=np.float64) -> Models:
    """Accept a Models handle or a host (nbins, nt) matrix (uploaded with storage
    matching its element type)."""
    if isinstance(models, Models):
        return models
    A = np.asarray(models)
    storage = "f32" if A.dtype == np.float32 else "f64"
    return Models(A, storage=storage)


__all__ = ["Context", "Models", "default_context", "as_models", "ptr", "_lib"]
