"""Host-side mirror of rta's plugin interfaces for the bbvh-cuda hot path.

The classes keep the reference's names, call order and argument meaning
(librta/raytrav.h, librta/cuda.h, bbvh-cuda/lbvh.h, bbvh-cuda/bbvh-cuda.h,
bbvh-cuda/main.cpp) and do their work through the C ABI of
include/rta_gb300.h.  Device memory comes from torch; there is no CPU path:
every operation runs the sm_103a kernels or fails.

    set = create_rt_set(triangles, w, h)      # bbvh-cuda/main.cpp:141-291
    set.rgen.setup(pos, dir, up, fovy)         # raytrav.h:338-343
    set.rt.ray_generator(set.rgen); set.rt.ray_bouncer(bouncer)
    set.rt.trace()                             # raytrav.h:411-421
    set.rt.timings                             # ms per bounce
"""
from __future__ import annotations

import argparse
import ctypes as C
import time

import numpy as np
import torch

from . import lib as L
from .scenes import TRI_FLOATS, tan_half_fovy

FLT_MAX = float(np.finfo(np.float32).max)
HIT_DTYPE = np.dtype([("t", "<f4"), ("beta", "<f4"), ("gamma", "<f4"), ("ref", "<u4")])


def _dev():
    if not torch.cuda.is_available():
        raise L.RtaError("a CUDA device is required (the GB300 path has no CPU fallback)")
    return torch.device("cuda")


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    return L.stream_handle(torch.cuda.current_stream())


# --------------------------------------------------------------------------- #
# triangle lists (librta/basic_types.h:57-63, librta/cuda-vec.h:234-243)       #
# --------------------------------------------------------------------------- #

class cuda_ftl:
    """Flat triangle list on the device: n records of cuda::simple_triangle."""

    def __init__(self, triangles):
        if isinstance(triangles, torch.Tensor):
            t = triangles
        else:
            t = torch.from_numpy(np.ascontiguousarray(triangles, np.float32).reshape(-1, TRI_FLOATS))
        self.triangle = t.to(_dev(), dtype=torch.float32).contiguous().view(-1, TRI_FLOATS)
        self.triangles = int(self.triangle.shape[0])


# --------------------------------------------------------------------------- #
# acceleration structure (bbvh-cuda/lbvh.h:13-34, bbvh-cuda/bbvh-cuda.h:29-73)  #
# --------------------------------------------------------------------------- #

class binary_lbvh:
    """The built tree.  triangle_ptr() is the Morton-ordered triangle array that
    triangle_intersection.ref indexes; index_buffer maps a Morton position to
    the input triangle id (lbvh.h:20-28)."""

    def __init__(self, ctor, tris_out: torch.Tensor):
        self.ctor = ctor
        self.view = L.LbvhView()
        L.check(L.load().rta_lbvh_get(ctor.handle, C.byref(self.view)), "rta_lbvh_get")
        self.triangle_data = tris_out
        self.n = int(self.view.n)

    # basic_acceleration_structure (raytrav.h:55-78)
    def identification(self) -> str:
        return "lbvh (gb300) based on the ba-sidaruck construction"

    def triangle_ptr(self) -> int:
        return self.triangle_data.data_ptr()

    def triangle_count(self) -> int:
        return self.n

    def canonical_triangle_ptr(self) -> np.ndarray:
        return self.triangle_data.cpu().numpy()

    def free_canonical_triangles(self, data) -> None:
        del data

    @property
    def index_buffer(self) -> np.ndarray:
        return device_view(self.view.index, self.n, "<u4").cpu().numpy().view(np.uint32)

    def node_data_2f4(self) -> np.ndarray:
        """The tree in the reference's 2F4 node layout, (2n-1, 8) float32."""
        out = torch.empty((2 * self.n - 1) * 8, dtype=torch.float32, device=_dev())
        L.check(L.load().rta_lbvh_to_2f4(C.byref(self.view), _ptr(out), _stream()), "rta_lbvh_to_2f4")
        return out.cpu().numpy().reshape(-1, 8)

    def codes(self) -> np.ndarray:
        wide = self.view.morton_bits == 63
        a = device_view(self.view.codes, self.n * (2 if wide else 1), "<u4").cpu().numpy()
        return a.view(np.uint64) if wide else a.view(np.uint32)

    def status(self) -> int:
        f = C.c_uint32(0)
        L.check(L.load().rta_lbvh_status(C.byref(self.view), _stream(), C.byref(f)), "rta_lbvh_status")
        return int(f.value)

    def dump_acceleration_structure(self, filename: str) -> None:
        """mamo text dump, the format of binary_bvh::dump_acceleration_structure
        (bbvh/bbvh.h:36-52), of the tree in the 2F4 node numbering."""
        with open(filename, "w") as f:
            f.write(format_bvh_dump(self.node_data_2f4()))

    def dump_primitives(self, filename: str) -> None:
        """mamo triangle dump (bbvh/bbvh.h:53-65) of the Morton-ordered records."""
        with open(filename, "w") as f:
            f.write(format_tri_dump(self.canonical_triangle_ptr()))


# --------------------------------------------------------------------------- #
# mamo text dumps: the reference writes them through std::ostream with its    #
# default float format (%g, 6 significant digits); these give the same text   #
# --------------------------------------------------------------------------- #

def _fmt(v) -> str:
    """One float as `std::ostream << float` prints it by default: %g of the
    value widened to double, "inf" / "-inf", and "nan" / "-nan" by the sign
    bit (as glibc prints NaNs)."""
    x = float(v)
    if x != x:
        return "-nan" if np.signbit(np.float32(v)) else "nan"
    return f"{x:g}"


def format_bvh_dump(nodes_2f4: np.ndarray) -> str:
    """binary_bvh::dump_acceleration_structure (bbvh/bbvh.h:36-52) of nodes in
    the 2F4 layout, (m, 8) float32: `i I|L box...` then `axis left right`
    for an inner node (the split axis of an LBVH node is 0, as bbvh_node's),
    `count tri tri+1 ...` for a leaf."""
    nodes = np.ascontiguousarray(nodes_2f4, np.float32).reshape(-1, 8)
    bits = nodes.view(np.uint32)
    out = [f"bvh\n{nodes.shape[0]}\n"]
    for i in range(nodes.shape[0]):
        w0, w1 = int(bits[i, 0]), int(bits[i, 1])
        box = " ".join(_fmt(v) for v in nodes[i, 2:8])
        if w0 & 1:
            out.append(f"{i} I {box} 0 {w0 >> 1} {w1}\n")
        else:
            el = w0 >> 1
            out.append(f"{i} L {box} {el}" + "".join(f" {(w1 + j) & 0xFFFFFFFF}" for j in range(el)) + "\n")
    return "".join(out)


def format_tri_dump(tris: np.ndarray) -> str:
    """binary_bvh::dump_primitives (bbvh/bbvh.h:53-65): index, positions a, b, c
    and normals na, nb, nc of each 104-byte record."""
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, TRI_FLOATS)
    out = [f"tri\n{t.shape[0]}\n"]
    for i in range(t.shape[0]):
        out.append(f"{i} " + " ".join(_fmt(v) for v in t[i, 0:18]) + "\n")
    return "".join(out)


def format_ray_dump(orig, dirs, maxt, w: int, h: int) -> str:
    """cam_ray_generator_shirley::dump_rays (librta/raytrav.h:353-366): per ray
    `y*w+x 2 origin direction 0 max_t`."""
    o = np.asarray(orig, np.float32).reshape(-1, 3)
    d = np.asarray(dirs, np.float32).reshape(-1, 3)
    m = np.asarray(maxt, np.float32).reshape(-1)
    out = [f"ray\n{int(w)} {int(h)}\n"]
    for i in range(int(w) * int(h)):
        out.append(f"{i} 2 {_fmt(o[i, 0])} {_fmt(o[i, 1])} {_fmt(o[i, 2])} "
                   f"{_fmt(d[i, 0])} {_fmt(d[i, 1])} {_fmt(d[i, 2])} 0 {_fmt(m[i])}\n")
    return "".join(out)


class _DevArray:
    """__cuda_array_interface__ wrapper of a raw device pointer (no ownership)."""

    def __init__(self, ptr: int, count: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (int(count),), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3, "strides": None}


def device_view(ptr, count: int, typestr: str = "<f4") -> torch.Tensor:
    """A torch view of `count` elements of device memory at `ptr` (no copy)."""
    p = ptr.value if isinstance(ptr, C.c_void_p) else ptr
    return torch.as_tensor(_DevArray(p, count, typestr), device=_dev())


class lbvh_constructor:
    """bbvh-cuda/lbvh.h:49-216.  Owns the device buffers (reused while the
    triangle count does not grow, lbvh.h:157-162)."""

    def __init__(self, morton_bits: int = 30, verbose: bool = False, keep_triangles: bool = True,
                 digit_bits: int = 8):
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.rta_lbvh_create(C.byref(h)), "rta_lbvh_create")
        self.handle = h
        L.check(self.lib.rta_lbvh_set_digit_bits(h, digit_bits), "rta_lbvh_set_digit_bits")
        self.morton_bits = morton_bits
        self.verbose = verbose
        self.keep_triangles = keep_triangles
        self.tris_out = None

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                self.lib.rta_lbvh_destroy(self.handle)
            except Exception:
                pass
            self.handle = None

    def identification(self) -> str:
        return "lbvh constructor (gb300)"

    def expects_host_triangles(self) -> bool:
        return False

    def build(self, ftl: cuda_ftl) -> binary_lbvh:
        n = ftl.triangles
        if self.keep_triangles:
            if self.tris_out is None or self.tris_out.shape[0] != n:
                self.tris_out = torch.empty((n, TRI_FLOATS), dtype=torch.float32, device=_dev())
        t0 = time.perf_counter()
        L.check(self.lib.rta_lbvh_build(self.handle, _ptr(ftl.triangle), n, self.morton_bits,
                                        _ptr(self.tris_out) if self.keep_triangles else C.c_void_p(0),
                                        _stream()), "rta_lbvh_build")
        bvh = binary_lbvh(self, self.tris_out)
        if self.verbose:
            torch.cuda.synchronize()
            print(f"Triangles: {n}  build {1e3 * (time.perf_counter() - t0):.3f} ms")
        return bvh


# --------------------------------------------------------------------------- #
# rays (librta/cuda.h:90-158) and bouncers (librta/cuda.h:193-266)             #
# --------------------------------------------------------------------------- #

class gpu_ray_generator:
    """Ray storage on the GPU: origin/direction float[3*w*h], max_t float[w*h]."""

    def __init__(self, w: int, h: int):
        self.w, self.h = int(w), int(h)
        dev = _dev()
        self.gpu_origin = torch.empty(3 * self.w * self.h, dtype=torch.float32, device=dev)
        self.gpu_direction = torch.empty(3 * self.w * self.h, dtype=torch.float32, device=dev)
        self.gpu_maxt = torch.empty(self.w * self.h, dtype=torch.float32, device=dev)

    def res_x(self):
        return self.w

    def dump_rays(self, filename: str) -> None:
        """mamo ray dump (librta/raytrav.h:353-366) of the rays on the device."""
        torch.cuda.synchronize()
        with open(filename, "w") as f:
            f.write(format_ray_dump(self.gpu_origin.cpu().numpy(), self.gpu_direction.cpu().numpy(),
                                    self.gpu_maxt.cpu().numpy(), self.w, self.h))

    def res_y(self):
        return self.h


class cam_ray_generator_shirley(gpu_ray_generator):
    """cuda::cam_ray_generator_shirley (librta/cuda.h:146-158)."""

    def __init__(self, res_x: int, res_y: int):
        super().__init__(res_x, res_y)
        self.aspect = np.float32(np.float32(res_x) / np.float32(res_y))
        self.position = np.zeros(3, np.float32)
        self.dir = np.array([0, 0, -1], np.float32)
        self.up = np.array([0, 1, 0], np.float32)
        self.fovy = 45.0

    def setup(self, position, direction, up, fovy) -> None:
        self.position = np.asarray(position, np.float32)
        self.dir = np.asarray(direction, np.float32)
        self.up = np.asarray(up, np.float32)
        self.fovy = float(fovy)

    def generate_rays(self) -> None:
        pos = (C.c_float * 3)(*self.position.tolist())
        vd = (C.c_float * 3)(*self.dir.tolist())
        up = (C.c_float * 3)(*self.up.tolist())
        L.check(L.load().rta_setup_shirley_rays(
            _ptr(self.gpu_direction), _ptr(self.gpu_origin), _ptr(self.gpu_maxt),
            float(tan_half_fovy(self.fovy)), float(self.aspect), self.w, self.h,
            vd, pos, up, FLT_MAX, _stream()), "rta_setup_shirley_rays")

    def identification(self) -> str:
        return "cuda version of the ray generator according to shirley."


class buffer_ray_generator(gpu_ray_generator):
    """Rays given as host or device arrays (raygen_with_buffer, librta/cuda.h:112-142)."""

    def __init__(self, orig, direction, maxt, w=None, h=1):
        n = int(np.asarray(maxt).shape[0]) if not isinstance(maxt, torch.Tensor) else int(maxt.shape[0])
        super().__init__(w or n, h if w else 1)
        self._src = (orig, direction, maxt)

    def generate_rays(self) -> None:
        o, d, m = self._src
        for dst, src in ((self.gpu_origin, o), (self.gpu_direction, d), (self.gpu_maxt, m)):
            t = src if isinstance(src, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(src, np.float32).reshape(-1))
            dst.copy_(t.reshape(-1), non_blocking=False)

    def identification(self) -> str:
        return "cuda raygen adaptor for host rays"


class gpu_ray_bouncer:
    """Device intersection buffer (librta/cuda.h:193-205)."""

    def __init__(self, w: int, h: int):
        self.w, self.h = int(w), int(h)
        self.gpu_last_intersection = torch.empty(self.w * self.h * 4, dtype=torch.float32, device=_dev())

    def new_pass(self) -> None:
        pass

    def intersections(self) -> np.ndarray:
        return self.gpu_last_intersection.cpu().numpy().view(HIT_DTYPE)


class primary_intersection_collector(gpu_ray_bouncer):
    """librta/cuda.h:208-220: primary rays only."""

    def trace_further_bounces(self) -> bool:
        return False

    def bounce(self) -> None:
        pass

    def identification(self) -> str:
        return "cuda primary intersection collector."


class host_frames:
    """rta_host_frames: frames whose rays and hits live in pinned host
    memory, pipelined so that one frame's copies overlap the neighbouring
    frames' traversal (two frames in flight)."""

    def __init__(self, max_rays: int):
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.rta_host_frames_create(C.byref(h), int(max_rays)), "rta_host_frames_create")
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                self.lib.rta_host_frames_destroy(self.handle)
            except Exception:
                pass
            self.handle = None

    def run(self, bvh, h_orig, h_dir, h_maxt, h_hits, h_bounce_hits, h_bounce_count, mode=L.TRACE_CIS,
            seed: int = 0, eps: float = 1e-4, nrays=None) -> None:
        n = int(h_maxt.numel() if nrays is None else nrays)
        L.check(self.lib.rta_host_frames_run(self.handle, C.byref(bvh.view), _ptr(h_orig), _ptr(h_dir),
                                             _ptr(h_maxt), n, _ptr(h_hits), _ptr(h_bounce_hits),
                                             _ptr(h_bounce_count), mode, seed, float(eps), _stream()),
                "rta_host_frames_run")


def write_png(filename: str, rgb: np.ndarray) -> None:
    """An (h, w, 3) uint8 image as an 8-bit RGB PNG (zlib from the standard
    library; rta's image<>::save_png writes the same pixels through png++)."""
    import struct
    import zlib
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + np.ascontiguousarray(rgb[y]).tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff)

    with open(filename, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


class direct_diffuse_illumination(primary_intersection_collector):
    """cuda::direct_diffuse_illumination (librta/cuda.h:247-266) with the
    lighting_collector shader (librta/raytrav.h:174-243).  The reference
    downloads every hit and shades on the host; here the shading runs on the
    device (rta_shade_lambert) and only the 8-bit image comes back, byte for
    byte the host shader's."""

    def __init__(self, w: int, h: int):
        super().__init__(w, h)
        self.lights = []
        self.triangles = None
        self.n_tris = 0
        self.image = torch.zeros(self.w * self.h * 3, dtype=torch.uint8, device=_dev())
        self._bg = None

    def triangle_ptr(self, tris: torch.Tensor) -> None:
        """The Morton-ordered 104-byte records the hits index (the AS's
        triangle_ptr(), i.e. lbvh_constructor(keep_triangles=True))."""
        self.triangles = tris
        self.n_tris = int(tris.numel() // TRI_FLOATS)

    def add_pointlight(self, at, col) -> None:
        self.lights.append([float(x) for x in at] + [float(x) for x in col])

    def reset(self, c) -> None:
        self._bg = np.asarray(c, np.float32)
        self._shade(False, only_reset=True)

    def shade(self, binary_result_only: bool = False) -> None:
        self._shade(binary_result_only)

    def _shade(self, binary: bool, only_reset: bool = False) -> None:
        lights = np.asarray(self.lights, np.float32).reshape(-1, 6)
        n = 0 if only_reset else lights.shape[0]
        bg = self._bg if only_reset else None
        L.check(L.load().rta_shade_lambert(_ptr(self.gpu_last_intersection), _ptr(self.triangles), self.n_tris,
                                           self.w, self.h, lights.ctypes.data_as(C.c_void_p) if n else None, n,
                                           int(bool(binary)), bg.ctypes.data_as(C.c_void_p) if bg is not None
                                           else None, _ptr(self.image), None, _stream()), "rta_shade_lambert")

    def pixels(self) -> np.ndarray:
        return self.image.cpu().numpy().reshape(self.h, self.w, 3)

    def save(self, filename: str) -> None:
        write_png(filename, self.pixels())

    def identification(self) -> str:
        return "direct_diffuse_illumination shaded on the device (gb300)"


class diffuse_bounce_collector(gpu_ray_bouncer):
    """Added bouncer: after the primary pass, one cosine-weighted diffuse
    bounce ray per hit is generated on the device and traced in the second
    pass; the bounce rays and hits stay on the device (rta_frame)."""

    def __init__(self, w: int, h: int, seed: int = 0, eps: float = 1e-4):
        super().__init__(w, h)
        self.seed, self.eps = int(seed), float(eps)
        self.lib = L.load()
        hnd = C.c_void_p()
        L.check(self.lib.rta_frame_create(C.byref(hnd), self.w * self.h), "rta_frame_create")
        self.handle = hnd
        self.frame = L.FrameView()
        L.check(self.lib.rta_frame_get(self.handle, C.byref(self.frame)), "rta_frame_get")
        self.passes = 0
        self.tracer = None

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                self.lib.rta_frame_destroy(self.handle)
            except Exception:
                pass
            self.handle = None

    def new_pass(self) -> None:
        self.passes = 0

    def trace_further_bounces(self) -> bool:
        return self.passes == 1

    def bounce(self) -> None:
        if self.passes == 0:
            t = self.tracer
            L.check(self.lib.rta_diffuse_bounce(self.handle, C.byref(t.bbvh.view), _ptr(t.raygen.gpu_origin),
                                                _ptr(t.raygen.gpu_direction), _ptr(self.gpu_last_intersection),
                                                self.w * self.h, self.seed, self.eps, _stream()),
                    "rta_diffuse_bounce")
        self.passes += 1

    def bounce_count(self) -> int:
        torch.cuda.current_stream().synchronize()
        return int(device_view(self.frame.count, 1, "<u4").cpu().numpy().view(np.uint32)[0])

    def identification(self) -> str:
        return "diffuse bounce collector (one cosine-weighted bounce, gb300)"


# --------------------------------------------------------------------------- #
# tracers (bbvh-cuda/bbvh-cuda.h:79-319, librta/raytrav.h:388-437)             #
# --------------------------------------------------------------------------- #

class bbvh_gpu_tracer:
    """gpu_raytracer + bbvh_gpu_tracer: the trace cycle of basic_raytracer and
    the acceleration_structure() re-binding contract (bbvh-cuda.h:89-92)."""

    mode = L.TRACE_CIS
    name = "cuda bbvh tracer."

    def __init__(self, gen, bvh, bouncer):
        self.raygen = gen
        self.bouncer = bouncer
        self.bbvh = bvh
        self.accel_struct = bvh
        self.timings = []
        self.lib = L.load()

    def identification(self) -> str:
        return self.name

    def supports_max_t(self) -> bool:
        return True

    def copy(self):
        c = type(self)(self.raygen, self.bbvh, self.bouncer)
        return c

    def ray_generator(self, rg) -> None:
        self.raygen = rg

    def ray_bouncer(self, rb) -> None:
        self.bouncer = rb
        if isinstance(rb, diffuse_bounce_collector):
            rb.tracer = self

    def acceleration_structure(self, as_=None):
        if as_ is None:
            return self.accel_struct
        self.bbvh = as_
        self.accel_struct = as_
        return None

    def prepare_trace(self) -> None:
        """reset_intersections on the buffer of this pass (cuda.h:301-303)."""
        b = self.bouncer
        buf = _ptr(b.gpu_last_intersection)
        if isinstance(b, diffuse_bounce_collector) and b.passes == 1:
            buf = C.c_void_p(b.frame.hits)   # the bounce pass's own hit buffer
        L.check(self.lib.rta_reset_intersections(buf, b.w, b.h, _stream()), "rta_reset_intersections")

    def trace_rays(self) -> float:
        """Kernel time of one pass in ms (CUDA events on the current stream)."""
        b = self.bouncer
        s = _stream()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        if isinstance(b, diffuse_bounce_collector) and b.passes == 1:
            f = b.frame
            rc = self.lib.rta_trace(C.byref(self.bbvh.view), C.c_void_p(f.orig), C.c_void_p(f.dir),
                                    C.c_void_p(f.maxt), 0, C.c_void_p(f.count), C.c_void_p(f.hits),
                                    self.mode, C.c_void_p(0), s)
        else:
            g = self.raygen
            rc = self.lib.rta_trace(C.byref(self.bbvh.view), _ptr(g.gpu_origin), _ptr(g.gpu_direction),
                                    _ptr(g.gpu_maxt), g.w * g.h, C.c_void_p(0),
                                    _ptr(b.gpu_last_intersection), self.mode, C.c_void_p(0), s)
        L.check(rc, "rta_trace")
        ev1.record()
        ev1.synchronize()
        return float(ev0.elapsed_time(ev1))

    def trace(self) -> None:
        """basic_raytracer::trace (raytrav.h:411-421)."""
        self.raygen.generate_rays()
        self.bouncer.new_pass()
        self.timings = []
        while True:
            self.prepare_trace()
            self.timings.append(self.trace_rays())
            self.bouncer.bounce()
            if not self.bouncer.trace_further_bounces():
                break


class bbvh_gpu_cis_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_CIS
    name = "cuda bbvh child-is tracer (gb300)."


class bbvh_gpu_dis_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_DIS
    name = "cuda bbvh tracer (gb300)."


class bbvh_gpu_cis_shadow_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_CIS | L.TRACE_SHADOW
    name = "cuda bbvh child-is shadow tracer (gb300)."


class bbvh_gpu_dis_shadow_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_DIS | L.TRACE_SHADOW
    name = "cuda bbvh shadow tracer (gb300)."


class bbvh_gpu_cis_ailabox_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_CIS | L.TRACE_AILA
    name = "cuda bbvh child-is tracer, aila box (gb300)."


class bbvh_gpu_dis_ailabox_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_DIS | L.TRACE_AILA
    name = "cuda bbvh tracer, aila box (gb300)."


class bbvh_gpu_cis_ailabox_shadow_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_CIS | L.TRACE_AILA | L.TRACE_SHADOW
    name = "cuda bbvh child-is shadow tracer, aila box (gb300)."


class bbvh_gpu_dis_ailabox_shadow_tracer(bbvh_gpu_tracer):
    mode = L.TRACE_DIS | L.TRACE_AILA | L.TRACE_SHADOW
    name = "cuda bbvh shadow tracer, aila box (gb300)."


# --------------------------------------------------------------------------- #
# plugin entry points (bbvh-cuda/main.cpp:17-291)                              #
# --------------------------------------------------------------------------- #

class Cmdline:
    def __init__(self):
        self.bvh_build = "median"
        self.bvh_trav = "cis"
        self.layout = "cpu"
        self.shadow_rays = False
        self.ailabox = False
        self.verbose = False
        self.morton_bits = 30


cmdline = Cmdline()
plugin_with_cuda_loaded = False


def description() -> str:
    return "a binary bvh ray tracer (gb300 lbvh)"


def initialize() -> None:
    global plugin_with_cuda_loaded
    plugin_with_cuda_loaded = True


def parse_cmdline(argv) -> int:
    """argp options of bbvh-cuda/main.cpp:40-51 (+ --morton-bits)."""
    p = argparse.ArgumentParser(prog="bbvh", add_help=True)
    p.add_argument("-v", "--verbose", action="store_true")
    p.add_argument("-b", "--bvh", default="median")
    p.add_argument("-l", "--layout", default="cpu")
    p.add_argument("-s", "--shadow", action="store_true")
    p.add_argument("-t", "--trav", default="cis")
    p.add_argument("-A", "--ailabox", action="store_true")
    p.add_argument("--morton-bits", type=int, default=30, choices=(30, 63))
    a = p.parse_args(list(argv[1:]) if argv else [])
    if a.trav not in ("dis", "cis"):
        raise SystemExit(f"Unknown bvh traversal scheme: {a.trav}")
    cmdline.verbose = a.verbose
    cmdline.bvh_build = "lbvh" if a.bvh == "lbvh" else "median"
    cmdline.layout = "2f4" if a.layout == "2f4" else "cpu"
    cmdline.shadow_rays = a.shadow
    cmdline.bvh_trav = a.trav
    cmdline.ailabox = a.ailabox
    cmdline.morton_bits = a.morton_bits
    return 0


class rt_set:
    """librta/librta.h:10-27."""

    def __init__(self):
        self.as_ = None
        self.ctor = None
        self.bouncer = None
        self.rt = None
        self.rgen = None

    def basic_rt(self):
        return self.rt

    def basic_as(self):
        return self.as_

    def basic_ctor(self):
        return self.ctor


_TRACERS = {
    (False, "dis", False): bbvh_gpu_dis_tracer, (False, "dis", True): bbvh_gpu_dis_shadow_tracer,
    (False, "cis", False): bbvh_gpu_cis_tracer, (False, "cis", True): bbvh_gpu_cis_shadow_tracer,
    (True, "dis", False): bbvh_gpu_dis_ailabox_tracer, (True, "dis", True): bbvh_gpu_dis_ailabox_shadow_tracer,
    (True, "cis", False): bbvh_gpu_cis_ailabox_tracer, (True, "cis", True): bbvh_gpu_cis_ailabox_shadow_tracer,
}


def create_rt_set(triangle_lists, w: int, h: int) -> rt_set:
    """bbvh-cuda/main.cpp:141-291.  Every -b/-l choice builds the LBVH on the
    GPU (the reference's 'median' builder is a CPU build, out of this path);
    the tracer class follows -t/-s/-A."""
    ftl = cuda_ftl(triangle_lists)
    ctor = lbvh_constructor(morton_bits=cmdline.morton_bits, verbose=cmdline.verbose)
    bvh = ctor.build(ftl)
    rt_cls = _TRACERS[(cmdline.ailabox, cmdline.bvh_trav, cmdline.shadow_rays)]
    s = rt_set()
    s.as_ = bvh
    s.ctor = ctor
    s.rt = rt_cls(None, bvh, None)
    s.rgen = cam_ray_generator_shirley(w, h)
    s.device_triangles = ftl
    return s
