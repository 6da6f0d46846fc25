"""ctypes binding of the C ABI in include/rta_gb300.h.

Device memory is handed over as raw pointers (for example ``tensor.data_ptr()``
of a CUDA torch tensor) and streams as raw ``cudaStream_t`` handles
(``torch.cuda.current_stream().cuda_stream``).  Loading fails loudly when the
library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librta_gb300.so")

OK = 0
ERR_INVALID, ERR_CUDA, ERR_DEVICE, ERR_NOMEM = -1, -2, -3, -4
DEV_STACK_OVERFLOW, DEV_SPIN_TIMEOUT, DEV_QUANT_WRAP, DEV_ZERO_EXTENT, DEV_ITER_LIMIT, DEV_BAD_LINK = 1, 2, 4, 8, 16, 32
TRACE_CIS, TRACE_DIS, TRACE_SHADOW, TRACE_AILA, TRACE_STATS = 0, 1, 2, 4, 8
LBVH_PASSES = 5

# every symbol include/rta_gb300.h declares
SYMBOLS = [
    "rta_last_error", "rta_lbvh_max_triangles", "rta_lbvh_create", "rta_lbvh_destroy",
    "rta_lbvh_reserve", "rta_lbvh_set_digit_bits", "rta_lbvh_build", "rta_lbvh_set_timing", "rta_lbvh_pass_ms",
    "rta_lbvh_get", "rta_lbvh_status", "rta_selftest_bounded_wait", "rta_lbvh_to_2f4",
    "rta_trace", "rta_setup_shirley_rays", "rta_reset_intersections", "rta_frame_create",
    "rta_frame_destroy", "rta_frame_get", "rta_diffuse_bounce", "rta_frame_run",
    "rta_frame_status", "rta_frame_set_timing", "rta_frame_trace_ms", "rta_host_frames_create", "rta_host_frames_destroy", "rta_host_frames_run",
    "rta_diffuse_bounce_noalloc", "rta_order_create", "rta_order_destroy",
    "rta_order_param_count", "rta_order_get_params", "rta_order_set_params", "rta_order_set_margin",
    "rta_order_get_margin", "rta_order_sample",
    "rta_order_sample_count", "rta_order_clear_samples", "rta_order_samples", "rta_order_gradient",
    "rta_order_train", "rta_trace_learned", "rta_trace_ideal_order",
    "rta_shade_lambert", "rta_batch_create", "rta_batch_destroy", "rta_batch_set_meshes", "rta_batch_build", "rta_batch_trace",
    "rta_batch_run", "rta_batch_mesh", "rta_batch_status", "rta_batch_get_params", "rta_batch_set_params",
    "rta_batch_autotune", "rta_batch_tune_key", "rta_tune_cache_lookup", "rta_tune_cache_store",
]
BOUNCE_NOALLOC_MAX_RAYS = 1 << 24


class RtaError(RuntimeError):
    pass


class LbvhView(C.Structure):
    """struct rta_lbvh"""
    _fields_ = [("nodes", C.c_void_p), ("root", C.c_void_p), ("tris", C.c_void_p),
                ("index", C.c_void_p), ("codes", C.c_void_p), ("parents", C.c_void_p),
                ("n", C.c_uint32), ("morton_bits", C.c_int32), ("status", C.c_void_p),
                ("ready", C.c_void_p)]


class FrameView(C.Structure):
    """struct rta_frame"""
    _fields_ = [("orig", C.c_void_p), ("dir", C.c_void_p), ("maxt", C.c_void_p),
                ("src", C.c_void_p), ("hits", C.c_void_p), ("count", C.c_void_p),
                ("capacity", C.c_uint32)]


class BatchParams(C.Structure):
    """struct rta_batch_params"""
    _fields_ = [("digit_bits", C.c_int32), ("fetch_idle", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("stack", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """The library at `path` with its argument types declared (cached)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RtaError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; "
                       f"g.build()'` (there is no CPU fallback)")
    L = C.CDLL(path)
    vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int32, C.c_float
    P = C.POINTER
    L.rta_last_error.restype = C.c_char_p
    L.rta_lbvh_max_triangles.restype = u32
    L.rta_lbvh_create.argtypes = [P(vp)]
    L.rta_lbvh_destroy.argtypes = [vp]
    L.rta_lbvh_reserve.argtypes = [vp, u32, i32]
    L.rta_lbvh_set_digit_bits.argtypes = [vp, i32]
    L.rta_lbvh_build.argtypes = [vp, vp, u32, i32, vp, vp]
    L.rta_lbvh_set_timing.argtypes = [vp, i32]
    L.rta_lbvh_pass_ms.argtypes = [vp, P(f32)]
    L.rta_lbvh_get.argtypes = [vp, P(LbvhView)]
    L.rta_lbvh_status.argtypes = [P(LbvhView), vp, P(u32)]
    L.rta_selftest_bounded_wait.argtypes = [vp, P(u32)]
    L.rta_lbvh_to_2f4.argtypes = [P(LbvhView), vp, vp]
    L.rta_trace.argtypes = [P(LbvhView), vp, vp, vp, u32, vp, vp, u32, vp, vp]
    L.rta_setup_shirley_rays.argtypes = [vp, vp, vp, f32, f32, i32, i32, vp, vp, vp, f32, vp]
    L.rta_reset_intersections.argtypes = [vp, u32, u32, vp]
    L.rta_frame_create.argtypes = [P(vp), u32]
    L.rta_frame_destroy.argtypes = [vp]
    L.rta_frame_get.argtypes = [vp, P(FrameView)]
    L.rta_diffuse_bounce.argtypes = [vp, P(LbvhView), vp, vp, vp, u32, u32, f32, vp]
    L.rta_frame_run.argtypes = [vp, P(LbvhView), vp, vp, vp, u32, vp, u32, u32, f32, vp]
    L.rta_frame_status.argtypes = [vp, vp, P(u32)]
    L.rta_frame_set_timing.argtypes = [vp, i32]
    L.rta_frame_trace_ms.argtypes = [vp, P(f32)]
    L.rta_host_frames_create.argtypes = [P(vp), u32]
    L.rta_host_frames_destroy.argtypes = [vp]
    L.rta_host_frames_run.argtypes = [vp, P(LbvhView), vp, vp, vp, u32, vp, vp, vp, u32, u32, f32, vp]
    L.rta_order_create.argtypes = [P(vp), u32, u32]
    L.rta_order_destroy.argtypes = [vp]
    L.rta_order_param_count.restype = u32
    L.rta_order_get_params.argtypes = [vp, vp]
    L.rta_order_set_params.argtypes = [vp, vp]
    L.rta_order_set_margin.argtypes = [vp, f32]
    L.rta_order_get_margin.argtypes = [vp, P(f32)]
    L.rta_order_sample.argtypes = [vp, P(LbvhView), vp, vp, vp, u32, vp, vp, vp]
    L.rta_order_sample_count.argtypes = [vp, P(u32)]
    L.rta_order_clear_samples.argtypes = [vp]
    L.rta_order_samples.argtypes = [vp, P(vp)]
    L.rta_order_gradient.argtypes = [vp, u32, u32, vp, vp]
    L.rta_order_train.argtypes = [vp, u32, u32, f32, vp, vp]
    L.rta_trace_learned.argtypes = [P(LbvhView), vp, vp, vp, vp, u32, vp, vp, vp, vp]
    L.rta_trace_ideal_order.argtypes = [P(LbvhView), vp, vp, vp, u32, vp, vp, vp, vp]
    L.rta_diffuse_bounce_noalloc.argtypes = [P(LbvhView), vp, vp, vp, u32, u32, f32, vp, vp, vp, vp,
                                             vp, vp, vp]
    L.rta_shade_lambert.argtypes = [vp, vp, u32, u32, u32, vp, u32, i32, vp, vp, vp, vp]
    L.rta_batch_create.argtypes = [P(vp)]
    L.rta_batch_destroy.argtypes = [vp]
    L.rta_batch_set_meshes.argtypes = [vp, u32, vp, vp]
    L.rta_batch_build.argtypes = [vp, vp, vp]
    L.rta_batch_trace.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.rta_batch_run.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.rta_batch_mesh.argtypes = [vp, u32, P(LbvhView)]
    L.rta_batch_status.argtypes = [vp, vp, P(u32)]
    L.rta_batch_get_params.argtypes = [vp, P(BatchParams)]
    L.rta_batch_set_params.argtypes = [vp, P(BatchParams)]
    L.rta_batch_autotune.argtypes = [vp, vp, vp, vp, vp, vp, C.c_char_p, i32, vp, P(BatchParams), P(f32)]
    L.rta_batch_tune_key.argtypes = [vp, C.c_char_p, u32]
    L.rta_tune_cache_lookup.argtypes = [C.c_char_p, C.c_char_p, P(BatchParams)]
    L.rta_tune_cache_store.argtypes = [C.c_char_p, C.c_char_p, P(BatchParams), f32]
    for name in SYMBOLS:
        if not hasattr(L, name):
            continue
        fn = getattr(L, name)
        if fn.restype is None or fn.restype is C.c_int:
            if name not in ("rta_last_error", "rta_lbvh_max_triangles", "rta_order_param_count"):
                fn.restype = C.c_int
    if path == LIB_PATH:
        _lib = L
    return L


def check(rc: int, what: str) -> None:
    if rc != OK:
        msg = load().rta_last_error().decode(errors="replace")
        raise RtaError(f"{what} failed with status {rc}: {msg}")


def stream_handle(stream) -> C.c_void_p:
    """Accepts None, an int handle or a torch.cuda.Stream."""
    if stream is None:
        return C.c_void_p(0)
    h = getattr(stream, "cuda_stream", stream)
    return C.c_void_p(int(h))
