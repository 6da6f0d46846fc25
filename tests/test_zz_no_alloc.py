"""rta_diffuse_bounce_noalloc: the bounce pass for callers that may not
allocate device memory (a renderer whose device memory belongs to its own
fixed-budget pool, or a frame loop that must not take cudaMalloc's implicit
device synchronisation between passes).

The entry point must give exactly what rta_diffuse_bounce gives (bounce
rays, their source rays and the count, bit for bit) on two calls in a row:
the second call reuses the shared scratch the first one left behind, so this
also checks that each call clears what must start at zero.  This file runs
last (its name sorts last) and passes alone in a fresh process or after the
other tests."""
import ctypes as C

import numpy as np
import pytest

from rta_gb300 import lib as L


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except ImportError:
        return True


def test_rejects_more_rays_than_the_scratch_holds():
    lib = L.load()
    view = L.LbvhView()
    view.tris, view.n = 16, 1
    fake = C.c_void_p(256)
    rc = lib.rta_diffuse_bounce_noalloc(C.byref(view), fake, fake, fake, L.BOUNCE_NOALLOC_MAX_RAYS + 1, 0,
                                        1e-4, fake, fake, fake, fake, fake, None, None)
    assert rc == L.ERR_INVALID
    assert b"exceed" in lib.rta_last_error()


@pytest.mark.skipif(not _no_gpu(), reason="fake pointers: only where no GPU can run the kernel")
def test_accepts_exactly_the_scratch_limit():
    """RTA_BOUNCE_NOALLOC_MAX_RAYS itself passes the size check: without a
    GPU the call then fails at the device lookup, not on the argument."""
    lib = L.load()
    view = L.LbvhView()
    view.tris, view.n = 16, 1
    fake = C.c_void_p(256)
    rc = lib.rta_diffuse_bounce_noalloc(C.byref(view), fake, fake, fake, L.BOUNCE_NOALLOC_MAX_RAYS, 0,
                                        1e-4, fake, fake, fake, fake, fake, None, None)
    assert rc == L.ERR_CUDA
    assert b"exceed" not in lib.rta_last_error()


@pytest.mark.gpu
def test_noalloc_bounce_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    from rta_gb300 import plugin as P
    from rta_gb300 import scenes as S

    lib = L.load()
    dev = torch.device("cuda")
    tris = S.terrain(128, 64, seed=21)
    ctor = P.lbvh_constructor(morton_bits=30)
    bvh = ctor.build(P.cuda_ftl(tris))
    stream = P._stream()

    def primary(w, h):
        cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=w, h=h)
        g = P.cam_ray_generator_shirley(w, h)
        g.setup(cam.pos, cam.dir, cam.up, cam.fovy)
        g.generate_rays()
        hits = torch.empty(4 * w * h, dtype=torch.float32, device=dev)
        L.check(lib.rta_reset_intersections(P._ptr(hits), w, h, stream), "reset")
        L.check(lib.rta_trace(C.byref(bvh.view), P._ptr(g.gpu_origin), P._ptr(g.gpu_direction),
                              P._ptr(g.gpu_maxt), w * h, None, P._ptr(hits), L.TRACE_CIS, None, stream),
                "trace")
        return g, hits

    def with_frame_ctx(g, hits, n, seed):
        fh = C.c_void_p()
        L.check(lib.rta_frame_create(C.byref(fh), n), "rta_frame_create")
        try:
            L.check(lib.rta_diffuse_bounce(fh, C.byref(bvh.view), P._ptr(g.gpu_origin),
                                           P._ptr(g.gpu_direction), P._ptr(hits), n, seed,
                                           np.float32(1e-4), stream), "rta_diffuse_bounce")
            f = L.FrameView()
            L.check(lib.rta_frame_get(fh, C.byref(f)), "rta_frame_get")
            torch.cuda.synchronize()
            cnt = int(P.device_view(f.count, 1, "<u4").cpu().numpy().view(np.uint32)[0])
            return (cnt, P.device_view(f.orig, 3 * cnt).cpu().numpy(),
                    P.device_view(f.dir, 3 * cnt).cpu().numpy(),
                    P.device_view(f.maxt, cnt).cpu().numpy(),
                    P.device_view(f.src, cnt, "<u4").cpu().numpy())
        finally:
            lib.rta_frame_destroy(fh)

    def without_alloc(g, hits, n, seed):
        oo = torch.empty(3 * n, dtype=torch.float32, device=dev)
        od = torch.empty(3 * n, dtype=torch.float32, device=dev)
        om = torch.empty(n, dtype=torch.float32, device=dev)
        src = torch.empty(n, dtype=torch.int32, device=dev)
        cnt = torch.full((1,), -1, dtype=torch.int32, device=dev)
        flags = torch.full((1,), -1, dtype=torch.int32, device=dev)
        L.check(lib.rta_diffuse_bounce_noalloc(C.byref(bvh.view), P._ptr(g.gpu_origin),
                                               P._ptr(g.gpu_direction), P._ptr(hits), n, seed,
                                               np.float32(1e-4), P._ptr(oo), P._ptr(od), P._ptr(om),
                                               P._ptr(src), P._ptr(cnt), P._ptr(flags), stream),
                "rta_diffuse_bounce_noalloc")
        torch.cuda.synchronize()
        assert int(flags.item()) == 0   # no look-back wait gave up
        c = int(cnt.item())
        return (c, oo[: 3 * c].cpu().numpy(), od[: 3 * c].cpu().numpy(), om[:c].cpu().numpy(),
                src[:c].cpu().numpy())

    # calls in a row, each smaller than the one before and with another seed;
    # the last is one partial tile (< 1024 rays), so the look-back words the
    # larger calls left beyond its range must not matter
    for (w, h), seed in (((320, 180), 3), ((160, 90), 4), ((40, 20), 5)):
        g, hits = primary(w, h)
        want = with_frame_ctx(g, hits, w * h, seed)
        got = without_alloc(g, hits, w * h, seed)
        assert want[0] > 0 and got[0] == want[0]
        for a, b in zip(got[1:], want[1:]):
            np.testing.assert_array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@pytest.mark.gpu
def test_noalloc_bounce_at_exactly_the_scratch_limit():
    """RTA_BOUNCE_NOALLOC_MAX_RAYS rays, all misses: the call uses every
    look-back word of the scratch and reports no bounce ray."""
    torch = pytest.importorskip("torch")
    from rta_gb300 import plugin as P
    from rta_gb300 import scenes as S

    lib = L.load()
    dev = torch.device("cuda")
    bvh = P.lbvh_constructor(morton_bits=30).build(P.cuda_ftl(S.terrain(8, 4, seed=1)))
    n = L.BOUNCE_NOALLOC_MAX_RAYS
    stream = P._stream()
    rays = torch.zeros(3 * n, dtype=torch.float32, device=dev)
    hits = torch.empty(4 * n, dtype=torch.float32, device=dev)
    L.check(lib.rta_reset_intersections(P._ptr(hits), n, 1, stream), "reset")
    oo = torch.empty(3 * n, dtype=torch.float32, device=dev)
    od = torch.empty(3 * n, dtype=torch.float32, device=dev)
    om = torch.empty(n, dtype=torch.float32, device=dev)
    src = torch.empty(n, dtype=torch.int32, device=dev)
    cnt = torch.full((1,), -1, dtype=torch.int32, device=dev)
    flags = torch.full((1,), -1, dtype=torch.int32, device=dev)
    L.check(lib.rta_diffuse_bounce_noalloc(C.byref(bvh.view), P._ptr(rays), P._ptr(rays), P._ptr(hits), n, 7,
                                           np.float32(1e-4), P._ptr(oo), P._ptr(od), P._ptr(om), P._ptr(src),
                                           P._ptr(cnt), P._ptr(flags), stream), "rta_diffuse_bounce_noalloc")
    torch.cuda.synchronize()
    assert int(cnt.item()) == 0 and int(flags.item()) == 0
