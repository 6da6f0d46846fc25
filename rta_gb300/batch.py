"""Batched multi-mesh LBVH build and trace over the C ABI (rta_batch_*).

Many independent meshes, each with its own tree and its own rays, built by
one pass sequence and traced by one persistent launch; `run` replays build +
trace as one CUDA graph, and `autotune` picks the launch parameters (sort
digit width, ray-fetch threshold, trace blocks per SM, stack depth) with a
JSON cache.  The reference has no batched path: it builds one mesh per
lbvh_constructor (bbvh-cuda/lbvh.h:153-211) and traces it with one launcher
call (bbvh-cuda/kernels.cu:1145-1338), which `sequential` reproduces mesh by
mesh for comparison.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import lib as L
from . import scenes as S
from .plugin import _dev, _ptr, _stream, binary_lbvh, cuda_ftl, lbvh_constructor


class mesh_lbvh(binary_lbvh):
    """One mesh's tree inside a batch, as a one-mesh view."""

    def __init__(self, batch: "Batch", mesh: int):
        self.ctor = batch
        self.view = L.LbvhView()
        L.check(batch.lib.rta_batch_mesh(batch.handle, mesh, C.byref(self.view)), "rta_batch_mesh")
        self.triangle_data = None
        self.n = int(self.view.n)


class Batch:
    """rta_batch: the meshes' trees, launch parameters and the run graph."""

    def __init__(self):
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.rta_batch_create(C.byref(h)), "rta_batch_create")
        self.handle = h
        self.meshes = 0

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                self.lib.rta_batch_destroy(self.handle)
            except Exception:
                pass
            self.handle = None

    def set_meshes(self, tri_offsets, ray_offsets) -> None:
        t = np.ascontiguousarray(tri_offsets, np.uint32)
        r = np.ascontiguousarray(ray_offsets, np.uint32)
        if t.shape != r.shape or t.ndim != 1 or t.shape[0] < 2:
            raise ValueError("offset arrays of meshes + 1 entries expected")
        L.check(self.lib.rta_batch_set_meshes(self.handle, t.shape[0] - 1, t.ctypes.data_as(C.c_void_p),
                                              r.ctypes.data_as(C.c_void_p)), "rta_batch_set_meshes")
        self.meshes = t.shape[0] - 1
        self.tri_offsets, self.ray_offsets = t.copy(), r.copy()

    def build(self, tris: torch.Tensor) -> None:
        L.check(self.lib.rta_batch_build(self.handle, _ptr(tris), _stream()), "rta_batch_build")

    def trace(self, orig, dirs, maxt, hits, stats=None) -> None:
        L.check(self.lib.rta_batch_trace(self.handle, _ptr(orig), _ptr(dirs), _ptr(maxt), _ptr(hits), _ptr(stats),
                                         _stream()), "rta_batch_trace")

    def run(self, tris, orig, dirs, maxt, hits) -> None:
        L.check(self.lib.rta_batch_run(self.handle, _ptr(tris), _ptr(orig), _ptr(dirs), _ptr(maxt), _ptr(hits),
                                       _stream()), "rta_batch_run")

    def mesh(self, m: int) -> mesh_lbvh:
        return mesh_lbvh(self, m)

    def status(self) -> int:
        f = C.c_uint32(0)
        L.check(self.lib.rta_batch_status(self.handle, _stream(), C.byref(f)), "rta_batch_status")
        return int(f.value)

    @property
    def params(self) -> dict:
        p = L.BatchParams()
        L.check(self.lib.rta_batch_get_params(self.handle, C.byref(p)), "rta_batch_get_params")
        return p.as_dict()

    @params.setter
    def params(self, d: dict) -> None:
        p = L.BatchParams(**{**self.params, **d})
        L.check(self.lib.rta_batch_set_params(self.handle, C.byref(p)), "rta_batch_set_params")

    def tune_key(self) -> str:
        buf = C.create_string_buffer(512)
        L.check(self.lib.rta_batch_tune_key(self.handle, buf, 512), "rta_batch_tune_key")
        return buf.value.decode()

    def autotune(self, tris, orig, dirs, maxt, hits, cache_path=None, reps: int = 5):
        """Returns (chosen parameters, median ms of one run; -1 when the cache
        supplied the choice)."""
        p = L.BatchParams()
        ms = C.c_float(0)
        L.check(self.lib.rta_batch_autotune(self.handle, _ptr(tris), _ptr(orig), _ptr(dirs), _ptr(maxt), _ptr(hits),
                                            cache_path.encode() if cache_path else None, reps, _stream(),
                                            C.byref(p), C.byref(ms)), "rta_batch_autotune")
        return p.as_dict(), float(ms.value)


def tune_cache_lookup(path: str, key: str):
    p = L.BatchParams()
    rc = L.load().rta_tune_cache_lookup(path.encode(), key.encode(), C.byref(p))
    return p.as_dict() if rc == L.OK else None


def tune_cache_store(path: str, key: str, params: dict, ms: float) -> None:
    p = L.BatchParams(**params)
    L.check(L.load().rta_tune_cache_store(path.encode(), key.encode(), C.byref(p), float(ms)),
            "rta_tune_cache_store")


class Workload:
    """A batch's inputs on the device: concatenated triangles and rays with
    their per-mesh offsets (rays of mesh m: primary first, then incoherent)."""

    def __init__(self, specs, tris_host, tri_offsets, ray_offsets, orig, dirs, maxt):
        self.specs = specs
        self.tris_host = tris_host
        self.tri_offsets, self.ray_offsets = tri_offsets, ray_offsets
        self.tris = torch.from_numpy(tris_host).to(_dev())
        self.orig, self.dirs, self.maxt = orig, dirs, maxt

    @property
    def n_tris(self) -> int:
        return int(self.tri_offsets[-1])

    @property
    def n_rays(self) -> int:
        return int(self.ray_offsets[-1])

    def mesh_tris(self, m: int) -> np.ndarray:
        return self.tris_host[self.tri_offsets[m]:self.tri_offsets[m + 1]]

    def mesh_rays(self, m: int):
        a, b = int(self.ray_offsets[m]), int(self.ray_offsets[m + 1])
        return self.orig[3 * a:3 * b], self.dirs[3 * a:3 * b], self.maxt[a:b]


def make_workload(specs) -> Workload:
    """Generates every mesh (host), uploads the triangles, and writes every
    mesh's rays into one device buffer: the primary rays by the camera kernel
    (rta_setup_shirley_rays) at the mesh's offset, the incoherent ones from the
    host."""
    lib = L.load()
    tris = [S.batch_mesh_triangles(s) for s in specs]
    tri_off = np.zeros(len(specs) + 1, np.uint32)
    tri_off[1:] = np.cumsum([t.shape[0] for t in tris])
    ray_off = np.zeros(len(specs) + 1, np.uint32)
    ray_off[1:] = np.cumsum([s.n_rays for s in specs])
    total = int(ray_off[-1])
    dev = _dev()
    orig = torch.empty(3 * total, dtype=torch.float32, device=dev)
    dirs = torch.empty(3 * total, dtype=torch.float32, device=dev)
    maxt = torch.empty(total, dtype=torch.float32, device=dev)
    esz = 4
    for m, s in enumerate(specs):
        a = int(ray_off[m])
        cam = s.cam
        vd = (C.c_float * 3)(*[float(x) for x in cam.dir])
        ps = (C.c_float * 3)(*[float(x) for x in cam.pos])
        up = (C.c_float * 3)(*[float(x) for x in cam.up])
        L.check(lib.rta_setup_shirley_rays(C.c_void_p(dirs.data_ptr() + 3 * a * esz),
                                           C.c_void_p(orig.data_ptr() + 3 * a * esz),
                                           C.c_void_p(maxt.data_ptr() + a * esz), float(cam.tan_half),
                                           float(cam.aspect), cam.w, cam.h, vd, ps, up, float(S.FLT_MAX),
                                           _stream()),
                "rta_setup_shirley_rays")
        o, d, mx = S.batch_incoherent_rays(s, tris[m])
        b = a + s.n_primary
        orig[3 * b:3 * (b + mx.shape[0])].copy_(torch.from_numpy(o))
        dirs[3 * b:3 * (b + mx.shape[0])].copy_(torch.from_numpy(d))
        maxt[b:b + mx.shape[0]].copy_(torch.from_numpy(mx))
    torch.cuda.synchronize()
    return Workload(specs, np.ascontiguousarray(np.concatenate(tris)), tri_off, ray_off, orig, dirs, maxt)


def sequential(work: Workload, hits: torch.Tensor, ctor: lbvh_constructor | None = None):
    """The per-mesh path: for each mesh one rta_lbvh_build and one rta_trace
    (the reference's one-constructor-per-mesh usage), into the same hit
    buffer layout as the batch."""
    lib = L.load()
    ctor = ctor or lbvh_constructor(morton_bits=30, keep_triangles=False)
    esz = 16
    for m in range(len(work.tri_offsets) - 1):
        a, b = int(work.tri_offsets[m]), int(work.tri_offsets[m + 1])
        L.check(lib.rta_lbvh_build(ctor.handle, C.c_void_p(work.tris.data_ptr() + a * 104), b - a, 30,
                                   C.c_void_p(0), _stream()), "rta_lbvh_build")
        ra, rb = int(work.ray_offsets[m]), int(work.ray_offsets[m + 1])
        if rb == ra:
            continue
        view = L.LbvhView()
        L.check(lib.rta_lbvh_get(ctor.handle, C.byref(view)), "rta_lbvh_get")
        hp = C.c_void_p(hits.data_ptr() + ra * esz)
        L.check(lib.rta_reset_intersections(hp, rb - ra, 1, _stream()), "rta_reset_intersections")
        L.check(lib.rta_trace(C.byref(view), C.c_void_p(work.orig.data_ptr() + 3 * ra * 4),
                              C.c_void_p(work.dirs.data_ptr() + 3 * ra * 4),
                              C.c_void_p(work.maxt.data_ptr() + ra * 4), rb - ra, C.c_void_p(0), hp, L.TRACE_CIS,
                              C.c_void_p(0), _stream()), "rta_trace")
    return ctor


__all__ = ["Batch", "mesh_lbvh", "Workload", "make_workload", "sequential", "tune_cache_lookup",
           "tune_cache_store", "cuda_ftl"]
