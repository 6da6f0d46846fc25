"""Learned child order for the child-is traversal.

A 14-32-32-1 network (BF16 weights, FP32 accumulation, tensor cores) picks
which child to visit first wherever the plain traversal hits both children
(the plain rule is nearer-entry-first, bbvh-cuda/kernels.cu:818-827).  It is
trained on decisions that the plain traversal itself records; the label of a
decision is the child whose subtree holds the ray's final closest hit.  Every
child closer than the current hit is still visited, so the closest hit is
unchanged; only which of two triangles at exactly the same t is reported can
differ.  A model is kept for a scene only when it lowers the mean number of
nodes plus triangles tested per ray on that scene (`keep_for_scene`).

Features of a decision (rows of 16, the last two zero):
  0-2   ray direction
  3-6   entry and exit distance of the left and right child, relative to the
        span [min entry, max exit] of the two
  7     depth / 32
  8-9   log2(triangles under the left / right child) / 25
  10    1 if a hit has been found, else 0
  11    the current hit distance relative to the span (clamped to [0, 1] in
        steps of 1/4 of the span), 1 without a hit
  12    is_leaf(left) - is_leaf(right)
  13    +1 if the plain rule picks the left child, else -1
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import lib as L
from .plugin import _dev, _ptr, _stream, device_view

SAMPLE_BYTES = 64


class OrderModel:
    """rta_order_model: network, Adam state and the recorded samples."""

    def __init__(self, max_samples: int = 1 << 24, seed: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.rta_order_create(C.byref(h), int(max_samples), int(seed)), "rta_order_create")
        self.handle = h
        self.max_samples = int(max_samples)

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                self.lib.rta_order_destroy(self.handle)
            except Exception:
                pass
            self.handle = None

    # ---- parameters ----
    def params(self) -> np.ndarray:
        p = np.empty(self.lib.rta_order_param_count(), np.float32)
        L.check(self.lib.rta_order_get_params(self.handle, p.ctypes.data_as(C.c_void_p)), "get_params")
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        L.check(self.lib.rta_order_set_params(self.handle, p.ctypes.data_as(C.c_void_p)), "set_params")

    def set_margin(self, margin: float) -> None:
        """The network overrides the plain order only where |logit| > margin."""
        L.check(self.lib.rta_order_set_margin(self.handle, np.float32(margin)), "rta_order_set_margin")

    def margin(self) -> float:
        m = C.c_float(0)
        L.check(self.lib.rta_order_get_margin(self.handle, C.byref(m)), "rta_order_get_margin")
        return float(m.value)

    # ---- samples ----
    def sample(self, bvh, orig, dirs, maxt, nrays=None, d_nrays=None) -> torch.Tensor:
        """Plain trace that records decisions; returns the hits (device)."""
        n = int(nrays if nrays is not None else maxt.numel())
        hits = torch.zeros(4 * n, dtype=torch.float32, device=_dev())
        L.check(self.lib.rta_reset_intersections(_ptr(hits), n, 1, _stream()), "reset")
        L.check(self.lib.rta_order_sample(self.handle, C.byref(bvh.view), _ptr(orig), _ptr(dirs), _ptr(maxt),
                                          0 if d_nrays is not None else n,
                                          C.c_void_p(d_nrays) if d_nrays is not None else None,
                                          _ptr(hits), _stream()), "rta_order_sample")
        return hits

    def sample_count(self) -> int:
        n = C.c_uint32(0)
        L.check(self.lib.rta_order_sample_count(self.handle, C.byref(n)), "sample_count")
        return int(n.value)

    def clear_samples(self) -> None:
        L.check(self.lib.rta_order_clear_samples(self.handle), "clear_samples")

    def samples(self, count=None) -> np.ndarray:
        """The first `count` sample records as raw 32-bit words (16 per sample)."""
        n = self.sample_count() if count is None else int(count)
        p = C.c_void_p()
        L.check(self.lib.rta_order_samples(self.handle, C.byref(p)), "samples")
        torch.cuda.synchronize()
        raw = device_view(p.value, n * SAMPLE_BYTES // 4, "<u4").cpu().numpy()
        return raw

    # ---- training ----
    def gradient(self, first: int, count: int):
        g = np.empty(self.lib.rta_order_param_count(), np.float32)
        loss = C.c_float(0)
        L.check(self.lib.rta_order_gradient(self.handle, first, count, g.ctypes.data_as(C.c_void_p),
                                            C.byref(loss)), "rta_order_gradient")
        return g, float(loss.value)

    def train(self, epochs: int = 2, batch: int = 1 << 16, lr: float = 2e-3) -> float:
        loss = C.c_float(0)
        L.check(self.lib.rta_order_train(self.handle, epochs, batch, np.float32(lr), C.byref(loss),
                                         _stream()), "rta_order_train")
        return float(loss.value)

    # ---- inference ----
    def trace(self, bvh, orig, dirs, maxt, stats: bool = False, nrays=None, d_nrays=None):
        n = int(nrays if nrays is not None else maxt.numel())
        hits = torch.zeros(4 * n, dtype=torch.float32, device=_dev())
        L.check(self.lib.rta_reset_intersections(_ptr(hits), n, 1, _stream()), "reset")
        st = torch.zeros(2 * n, dtype=torch.int32, device=_dev()) if stats else None
        L.check(self.lib.rta_trace_learned(C.byref(bvh.view), self.handle, _ptr(orig), _ptr(dirs), _ptr(maxt),
                                           0 if d_nrays is not None else n,
                                           C.c_void_p(d_nrays) if d_nrays is not None else None,
                                           _ptr(hits), _ptr(st), _stream()), "rta_trace_learned")
        return (hits, st) if stats else hits


def plain_trace(bvh, orig, dirs, maxt, stats: bool = False):
    lib = L.load()
    n = int(maxt.numel())
    hits = torch.zeros(4 * n, dtype=torch.float32, device=_dev())
    L.check(lib.rta_reset_intersections(_ptr(hits), n, 1, _stream()), "reset")
    st = torch.zeros(2 * n, dtype=torch.int32, device=_dev()) if stats else None
    mode = L.TRACE_CIS | (L.TRACE_STATS if stats else 0)
    L.check(lib.rta_trace(C.byref(bvh.view), _ptr(orig), _ptr(dirs), _ptr(maxt), n, None, _ptr(hits), mode,
                          _ptr(st), _stream()), "rta_trace")
    return (hits, st) if stats else hits


def ideal_trace(bvh, orig, dirs, maxt, known_hits, stats: bool = False):
    """Trace with the ideal child order taken from `known_hits` (the closest
    hits of an earlier trace): the bound on what a learned order can gain."""
    lib = L.load()
    n = int(maxt.numel())
    hits = torch.zeros(4 * n, dtype=torch.float32, device=_dev())
    L.check(lib.rta_reset_intersections(_ptr(hits), n, 1, _stream()), "reset")
    st = torch.zeros(2 * n, dtype=torch.int32, device=_dev()) if stats else None
    L.check(lib.rta_trace_ideal_order(C.byref(bvh.view), _ptr(orig), _ptr(dirs), _ptr(maxt), n, _ptr(known_hits),
                                      _ptr(hits), _ptr(st), _stream()), "rta_trace_ideal_order")
    return (hits, st) if stats else hits


def work_per_ray(stats: torch.Tensor) -> float:
    """Mean nodes + triangles tested per ray."""
    s = stats.view(-1, 2).to(torch.float64)
    return float(s.sum(1).mean())


MARGINS = (0.0, 0.5, 1.0, 2.0, 4.0, 8.0, 16.0, float("inf"))


def choose_margin(model: OrderModel, bvh, orig, dirs, maxt, candidates=MARGINS) -> dict:
    """Sets the confidence margin (rta_order_set_margin) that gives the least
    mean nodes + triangles tested per ray on the given rays, which should be
    rays of the training scenes.  An infinite margin is the plain order, so
    the choice never does worse than plain on these rays; of equal results
    the larger margin (closer to plain) wins."""
    _, sp = plain_trace(bvh, orig, dirs, maxt, stats=True)
    plain = work_per_ray(sp)
    best_m, best_w, table = float("inf"), plain, {}
    for mg in candidates:
        if mg == float("inf"):
            table["inf"] = plain
            continue
        model.set_margin(mg)
        _, sl = model.trace(bvh, orig, dirs, maxt, stats=True)
        w = work_per_ray(sl)
        table[repr(mg)] = w
        if w < best_w or (w == best_w and mg > best_m):
            best_m, best_w = mg, w
    # an infinite choice is FLT_MAX, which runs the plain kernel (no network)
    model.set_margin(float(np.finfo(np.float32).max) if best_m == float("inf") else best_m)
    return {"margin": best_m, "work_per_ray": best_w, "plain_work_per_ray": plain, "tried": table}


def keep_for_scene(model: OrderModel, bvh, orig, dirs, maxt) -> dict:
    """Per-scene keep/reject: the learned order is kept only where it lowers
    the mean nodes + triangles tested per ray (plain order is the fallback)."""
    _, sp = plain_trace(bvh, orig, dirs, maxt, stats=True)
    _, sl = model.trace(bvh, orig, dirs, maxt, stats=True)
    wp, wl = work_per_ray(sp), work_per_ray(sl)
    return {"plain_work_per_ray": wp, "learned_work_per_ray": wl, "keep": wl < wp}
