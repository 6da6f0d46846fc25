"""ctypes front of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` as
the checker and by ``bench.py``'s CPU-baseline leg.  The product never imports
this module.

Arrays are numpy; triangles are (n, 26) float32 records in the reference's
``cuda::simple_triangle`` layout (librta/cuda-vec.h:30-37).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

CIS, DIS, SHADOW, AILA = 0, 1, 2, 4
FLAG_WRAP, FLAG_NONFINITE, FLAG_CODE0_RACE = 1, 2, 4
HIT_DTYPE = np.dtype([("t", "<f4"), ("beta", "<f4"), ("gamma", "<f4"), ("ref", "<u4")])

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _setup(_lib)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _setup(L):
    vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int, C.c_float
    L.orc_lbvh_build.argtypes = [vp, u32, i32, vp, vp, vp, vp, vp, vp]
    L.orc_lbvh_build.restype = i32
    L.orc_permute.argtypes = [vp, vp, u32, vp]
    L.orc_trace.argtypes = [vp, vp, vp, vp, vp, u32, i32, i32, vp, vp, i32]
    L.orc_trace.restype = i32
    L.orc_shirley_rays.argtypes = [vp, vp, vp, f32, f32, i32, i32, vp, vp, vp, f32]
    L.orc_reset_hits.argtypes = [vp, u32]
    L.orc_diffuse_bounce.argtypes = [vp, vp, vp, vp, u32, u32, f32, vp, vp, vp, vp]
    L.orc_diffuse_bounce.restype = u32
    L.orc_uniform.argtypes = [u32, u32]
    L.orc_uniform.restype = f32
    L.orc_cos_sin_2pi.argtypes = [f32, vp, vp]
    L.orc_bbvh_build.argtypes = [vp, u32, vp, vp, u32]
    L.orc_bbvh_build.restype = C.c_int64
    L.orc_bbvh_trace_cis.argtypes = [vp, vp, vp, vp, vp, u32, vp, i32]
    L.orc_bbvh_trace_cis.restype = i32
    L.orc_intersect_aabb.argtypes = [vp, vp, vp, vp, vp]
    L.orc_intersect_aabb.restype = i32
    L.orc_shade_lambert.argtypes = [vp, vp, u32, u32, vp, u32, i32, vp, vp]


class LBVH:
    """Result of :func:`lbvh_build` (reference layout)."""

    def __init__(self, codes, ids, nodes, scene, scale, flags, n, bits):
        self.codes, self.ids, self.nodes = codes, ids, nodes
        self.scene, self.scale, self.flags = scene, scale, flags
        self.n, self.bits = n, bits


def lbvh_build(tris: np.ndarray, bits: int = 30) -> LBVH:
    """K1-K6 of bbvh-cuda/lbvh-kernels.cu; nodes in the 2F4 layout (2n-1, 8) float32."""
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 26)
    n = tris.shape[0]
    codes = np.empty(n, np.uint64)
    ids = np.empty(n, np.uint32)
    nodes = np.empty((2 * n - 1, 8), np.float32)
    scene = np.empty(6, np.float32)
    scale = np.empty(3, np.float32)
    flags = np.zeros(1, np.uint32)
    rc = lib().orc_lbvh_build(_p(tris), n, bits, _p(codes), _p(ids), _p(nodes), _p(scene),
                              _p(scale), _p(flags))
    if rc != 0:
        raise ValueError(f"orc_lbvh_build failed ({rc})")
    return LBVH(codes, ids, nodes, scene, scale, int(flags[0]), n, bits)


def permute(tris: np.ndarray, ids: np.ndarray) -> np.ndarray:
    tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 26)
    out = np.empty_like(tris)
    lib().orc_permute(_p(tris), _p(np.ascontiguousarray(ids, np.uint32)), tris.shape[0], _p(out))
    return out


def trace(nodes, tris_sorted, orig, dirs, maxt, mode=CIS, stack_limit=256, hits=None,
          stats=False, threads=0):
    """Traces rays through a reference-layout BVH; returns (hits, stats|None, overflow)."""
    nodes = np.ascontiguousarray(nodes, np.float32)
    tris_sorted = np.ascontiguousarray(tris_sorted, np.float32)
    orig = np.ascontiguousarray(orig, np.float32).reshape(-1)
    dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1)
    maxt = np.ascontiguousarray(maxt, np.float32).reshape(-1)
    nr = maxt.shape[0]
    if hits is None:
        hits = reset_hits(nr)
    else:
        hits = np.array(hits, dtype=HIT_DTYPE, copy=True)
    st = np.zeros((nr, 2), np.uint32) if stats else None
    rc = lib().orc_trace(_p(nodes), _p(tris_sorted), _p(orig), _p(dirs), _p(maxt), nr, mode,
                         stack_limit, _p(hits), _p(st), threads)
    return hits, st, rc != 0


def reset_hits(n: int) -> np.ndarray:
    h = np.zeros(n, HIT_DTYPE)
    lib().orc_reset_hits(_p(h), n)
    return h


def shirley_rays(tan_half_fovy, aspect, w, h, view_dir, pos, up, maxt=np.finfo(np.float32).max):
    dirs = np.empty(3 * w * h, np.float32)
    orgs = np.empty(3 * w * h, np.float32)
    mt = np.empty(w * h, np.float32)
    vd = np.asarray(view_dir, np.float32)
    ps = np.asarray(pos, np.float32)
    u = np.asarray(up, np.float32)
    lib().orc_shirley_rays(_p(dirs), _p(orgs), _p(mt), float(tan_half_fovy), float(aspect), w, h,
                           _p(vd), _p(ps), _p(u), float(maxt))
    return orgs, dirs, mt


def diffuse_bounce(tris_sorted, orig, dirs, hits, seed, eps=1e-4):
    tris_sorted = np.ascontiguousarray(tris_sorted, np.float32)
    orig = np.ascontiguousarray(orig, np.float32).reshape(-1)
    dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1)
    hits = np.ascontiguousarray(hits, HIT_DTYPE)
    nr = hits.shape[0]
    oo = np.empty(3 * nr, np.float32)
    od = np.empty(3 * nr, np.float32)
    om = np.empty(nr, np.float32)
    src = np.empty(nr, np.uint32)
    m = lib().orc_diffuse_bounce(_p(tris_sorted), _p(orig), _p(dirs), _p(hits), nr, seed,
                                 float(eps), _p(oo), _p(od), _p(om), _p(src))
    return oo[:3 * m], od[:3 * m], om[:m], src[:m]


def shade_lambert(tris_sorted, hits, w, h, lights, binary=False, bg=None, img=None):
    """lighting_collector::reset + ::shade (librta/raytrav.h:186-233); returns
    the (h, w, 3) uint8 image.  lights: (k, 6) position xyz + colour rgb."""
    tris_sorted = np.ascontiguousarray(tris_sorted, np.float32)
    hits = np.ascontiguousarray(hits, HIT_DTYPE)
    lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 6)
    out = np.zeros((h, w, 3), np.uint8) if img is None else np.array(img, np.uint8, copy=True)
    bgp = None if bg is None else np.ascontiguousarray(bg, np.float32)
    lib().orc_shade_lambert(_p(tris_sorted), _p(hits), w, h, _p(lights), lights.shape[0], int(bool(binary)),
                            None if bgp is None else _p(bgp), _p(out))
    return out


def uniform(seed: int, index: int) -> float:
    return float(lib().orc_uniform(seed, index))


def cos_sin_2pi(u: float):
    c = np.zeros(1, np.float32)
    s = np.zeros(1, np.float32)
    lib().orc_cos_sin_2pi(float(u), _p(c), _p(s))
    return float(c[0]), float(s[0])


def bbvh_build(tris: np.ndarray):
    """Spatial-median CPU bbvh (bbvh/bbvh.h:206-277). Returns (nodes, leaf-ordered tris)."""
    work = np.array(tris, dtype=np.float32, copy=True).reshape(-1, 26)
    n = work.shape[0]
    out = np.empty_like(work)
    max_nodes = 2 * n + 8
    nodes = np.empty((max_nodes, 8), np.float32)
    cnt = lib().orc_bbvh_build(_p(work), n, _p(out), _p(nodes), max_nodes)
    if cnt < 0:
        raise ValueError(f"orc_bbvh_build failed ({cnt})")
    return nodes[:cnt].copy(), out


def bbvh_trace_cis(nodes, tris, orig, dirs, maxt, threads=0):
    nodes = np.ascontiguousarray(nodes, np.float32)
    tris = np.ascontiguousarray(tris, np.float32)
    orig = np.ascontiguousarray(orig, np.float32).reshape(-1)
    dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1)
    maxt = np.ascontiguousarray(maxt, np.float32).reshape(-1)
    nr = maxt.shape[0]
    hits = np.zeros(nr, HIT_DTYPE)
    lib().orc_bbvh_trace_cis(_p(nodes), _p(tris), _p(orig), _p(dirs), _p(maxt), nr, _p(hits),
                             threads)
    return hits


# --------------------------------------------------------------------------- #
# child-order network (checker of the tensor-core training kernels)            #
# --------------------------------------------------------------------------- #

MLP_PARAMS = 32 * 16 + 32 + 32 * 32 + 32 + 32 + 1
SAMPLE_DTYPE = np.dtype([("x", "<u2", 16), ("ray", "<u4"), ("lfirst", "<u4"), ("lsize", "<u4"),
                         ("rfirst", "<u4"), ("rsize", "<u4"), ("label", "<f4"), ("weight", "<f4"),
                         ("pad", "<u4")])


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even) -> float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_bits_to_f32(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, np.uint32) << 16).view(np.float32)


def mlp_unpack(params):
    p = np.asarray(params, np.float64)
    o = 0
    w1 = p[o:o + 512].reshape(32, 16); o += 512
    b1 = p[o:o + 32]; o += 32
    w2 = p[o:o + 1024].reshape(32, 32); o += 1024
    b2 = p[o:o + 32]; o += 32
    w3 = p[o:o + 32]; o += 32
    b3 = p[o]
    return w1, b1, w2, b2, w3, b3


def mlp_logits(params, x):
    """Forward pass with the kernels' rounding points: bf16 weights, inputs
    and hidden activations, accumulation in (here: double) precision."""
    w1, b1, w2, b2, w3, b3 = mlp_unpack(params)
    r = lambda a: bf16_round(np.asarray(a, np.float32)).astype(np.float64)  # noqa: E731
    z1 = r(x) @ r(w1).T + b1
    h1 = r(np.maximum(z1, 0))
    z2 = h1 @ r(w2).T + b2
    h2 = r(np.maximum(z2, 0))
    return h2 @ r(w3) + b3


def mlp_gradient(params, x, label, weight, scale):
    """Gradient of scale * sum(weight * BCE(logit, label)) and the weighted
    loss sum, restating k_mlp_grad (rta_gb300/csrc/learn.cu) in float64."""
    w1, b1, w2, b2, w3, b3 = mlp_unpack(params)
    r = lambda a: bf16_round(np.asarray(a, np.float32)).astype(np.float64)  # noqa: E731
    x = r(x)
    label = np.asarray(label, np.float64)
    weight = np.asarray(weight, np.float64)
    z1 = x @ r(w1).T + b1
    h1 = r(np.maximum(z1, 0))
    z2 = h1 @ r(w2).T + b2
    h2 = r(np.maximum(z2, 0))
    y = h2 @ r(w3) + b3
    p = 1.0 / (1.0 + np.exp(-y))
    dy = (p - label) * weight * scale
    loss = float(np.sum(weight * (np.maximum(y, 0) - y * label + np.log1p(np.exp(-np.abs(y))))))
    g_b3 = dy.sum()
    g_w3 = dy @ h2
    dz2 = (z2 > 0) * (dy[:, None] * r(w3)[None, :])
    g_b2 = dz2.sum(0)
    dz2b = r(dz2)
    g_w2 = dz2b.T @ h1
    dh1 = dz2b @ r(w2)
    dz1 = (z1 > 0) * dh1
    g_b1 = dz1.sum(0)
    g_w1 = r(dz1).T @ x
    grad = np.concatenate([g_w1.ravel(), g_b1, g_w2.ravel(), g_b2, g_w3, [g_b3]])
    return grad, loss
