"""GPU parity: the sm_103a build and traversal, called through the C ABI,
against the golden fixtures made by the reference's own code and against the
CPU oracle.  Everything is compared bit for bit: Morton codes, sorted ids,
every word of the 2F4 node array, the camera rays, and t / beta / gamma / ref
of every hit."""
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402
from rta_gb300 import lib as L  # noqa: E402
from rta_gb300 import plugin as P  # noqa: E402
from rta_gb300 import scenes as S  # noqa: E402

MODES = {"cis": L.TRACE_CIS, "dis": L.TRACE_DIS, "shadow_cis": L.TRACE_CIS | L.TRACE_SHADOW,
         "shadow_dis": L.TRACE_DIS | L.TRACE_SHADOW, "cis_aila": L.TRACE_CIS | L.TRACE_AILA,
         "dis_aila": L.TRACE_DIS | L.TRACE_AILA}
ORC = {"cis": O.CIS, "dis": O.DIS, "shadow_cis": O.CIS | O.SHADOW, "shadow_dis": O.DIS | O.SHADOW,
       "cis_aila": O.CIS | O.AILA, "dis_aila": O.DIS | O.AILA}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def records(pos):
    p = np.asarray(pos, np.float32).reshape(-1, 3, 3)
    return S._records(p[:, 0], p[:, 1], p[:, 2])


def gpu_build(tris, bits=30):
    ctor = P.lbvh_constructor(morton_bits=bits)
    bvh = ctor.build(P.cuda_ftl(tris))
    bvh._ctor_ref = ctor   # keep the buffers alive with the view
    return bvh


def gpu_trace(bvh, orig, dirs, maxt, mode, hits_init=None, stats=False):
    dev = torch.device("cuda")
    o = torch.from_numpy(np.ascontiguousarray(orig, np.float32).reshape(-1)).to(dev)
    d = torch.from_numpy(np.ascontiguousarray(dirs, np.float32).reshape(-1)).to(dev)
    m = torch.from_numpy(np.ascontiguousarray(maxt, np.float32).reshape(-1)).to(dev)
    n = m.shape[0]
    if hits_init is None:
        hits_init = O.reset_hits(n)
    h = torch.from_numpy(np.ascontiguousarray(hits_init).view(np.float32).reshape(-1).copy()).to(dev)
    st = torch.zeros(2 * n, dtype=torch.int32, device=dev) if stats else None
    import ctypes as C
    L.check(L.load().rta_trace(C.byref(bvh.view), P._ptr(o), P._ptr(d), P._ptr(m), n, C.c_void_p(0),
                               P._ptr(h), mode | (L.TRACE_STATS if stats else 0), P._ptr(st),
                               P._stream()), "rta_trace")
    torch.cuda.synchronize()
    out = h.cpu().numpy().view(O.HIT_DTYPE)
    if stats:
        return out, st.cpu().numpy().view(np.uint32).reshape(-1, 2)
    return out


def assert_hits_equal(a, b):
    for f in ("t", "beta", "gamma"):
        np.testing.assert_array_equal(a[f].view(np.uint32), b[f].view(np.uint32), err_msg=f)
    valid = a["t"] != np.float32(S.FLT_MAX)
    np.testing.assert_array_equal(a["ref"][valid], b["ref"][valid], err_msg="ref")


def assert_build_equals(bvh, codes, ids, nodes):
    np.testing.assert_array_equal(bvh.codes(), codes)
    np.testing.assert_array_equal(bvh.index_buffer, ids)
    np.testing.assert_array_equal(bvh.node_data_2f4().view(np.uint32), np.asarray(nodes).view(np.uint32))
    assert bvh.status() & ~(L.DEV_QUANT_WRAP | L.DEV_ZERO_EXTENT) == 0


# --------------------------------------------------------------------------- #
# LBVH                                                                         #
# --------------------------------------------------------------------------- #

@pytest.mark.parametrize("case", ["n1", "n2", "n3", "n7", "dup64", "rand100", "clump",
                                  "terrain16x8", "clusters4x64", "sphere"])
def test_build_matches_reference_golden(golden_dir, case):
    z = np.load(os.path.join(golden_dir, "lbvh_cases.npz"))
    bvh = gpu_build(records(z[f"{case}/pos"]), 30)
    assert_build_equals(bvh, z[f"{case}/codes"], z[f"{case}/ids"], z[f"{case}/nodes"])


@pytest.mark.parametrize("scene,bits", [("terrain", 30), ("clusters", 30), ("clusters", 63),
                                        ("terrain", 63)])
def test_build_matches_oracle(scene, bits):
    tris = S.terrain(256, 128, seed=2) if scene == "terrain" else S.clusters(32, 2048, seed=3)
    lb = O.lbvh_build(tris, bits)
    bvh = gpu_build(tris, bits)
    codes = lb.codes if bits == 63 else lb.codes.astype(np.uint32)
    assert_build_equals(bvh, codes, lb.ids, lb.nodes)
    # the Morton-ordered 104-byte records the AS exposes (lbvh-kernels.cu:557-578)
    np.testing.assert_array_equal(bvh.canonical_triangle_ptr().view(np.uint32),
                                  O.permute(tris, lb.ids).view(np.uint32))


@pytest.mark.parametrize("n", [255, 256, 257, 511, 513, 65535, 65536, 65537, 70001])
def test_build_at_refit_segment_and_group_borders(n):
    """The refit unions boxes over 256-leaf segments and 256-segment groups:
    triangle counts just below, at and above those borders (a last segment of
    one leaf, a last group of one segment) give the oracle's tree.  Every
    fourth triangle repeats its predecessor, so equal codes collapse across
    the borders too."""
    tris = S.clusters(1, n, seed=n)
    tris[3::4, :9] = tris[2:-1:4, :9][: len(tris[3::4])]
    for bits in (30, 63):
        lb = O.lbvh_build(tris, bits)
        bvh = gpu_build(tris, bits)
        codes = lb.codes if bits == 63 else lb.codes.astype(np.uint32)
        assert_build_equals(bvh, codes, lb.ids, lb.nodes)


@pytest.mark.parametrize("bits", [30, 63])
def test_build_signed_zero_ties_match_the_oracle(bits):
    """Box unions of equal values that differ in sign (-0.0 against +0.0):
    the oracle's sequential climb keeps the left child's value; the range
    refit keeps the leftmost leaf's, the same bits for every node."""
    tris = S.terrain(64, 32, seed=9)
    pos = tris[:, :9]
    zero = pos == 0.0
    assert zero.any()
    flip = np.zeros_like(zero)
    flip[1::2] = True   # every other triangle's zero coordinates become -0.0
    pos[zero & flip] = np.float32(-0.0)
    assert np.signbit(pos[zero]).any() and (~np.signbit(pos[zero])).any()
    lb = O.lbvh_build(tris, bits)
    bvh = gpu_build(tris, bits)
    codes = lb.codes if bits == 63 else lb.codes.astype(np.uint32)
    assert_build_equals(bvh, codes, lb.ids, lb.nodes)


@pytest.mark.parametrize("digit_bits", [9, 10, 11])
@pytest.mark.parametrize("bits", [30, 63])
def test_sort_digit_width_gives_the_same_tree(digit_bits, bits):
    """The stable LSD sort gives one order whatever its digit width (an odd
    number of passes leaves the result in the second buffer pair)."""
    tris = S.clusters(32, 2048, seed=5)
    lb = O.lbvh_build(tris, bits)
    ctor = P.lbvh_constructor(morton_bits=bits, digit_bits=digit_bits)
    bvh = ctor.build(P.cuda_ftl(tris))
    codes = lb.codes if bits == 63 else lb.codes.astype(np.uint32)
    assert_build_equals(bvh, codes, lb.ids, lb.nodes)


def _skewed_scene(kind, n, seed):
    """Triangle sets whose sort digits are badly skewed: `clump` puts all but
    every 997th triangle on one centroid (almost every key equal, so every
    pass sends nearly a whole tile to one digit), `two` splits them between
    two tiny far-apart clumps (two digits per pass), `ramp` repeats each of
    a few hundred positions in runs that straddle the 4096-key tiles."""
    rng = np.random.default_rng(seed)
    if kind == "clump":
        pos = np.tile(rng.uniform(-1, 1, 9), (n, 1))
        pos[::997] = rng.uniform(-1, 1, (len(pos[::997]), 9))
    elif kind == "two":
        a, b = rng.uniform(-1, 1, 9), rng.uniform(-1, 1, 9) + 50.0
        pos = np.where((np.arange(n) % 3 == 0)[:, None], a, b) + rng.normal(0, 1e-6, (n, 9))
    else:
        base = rng.uniform(-1, 1, (331, 9))
        pos = base[(np.arange(n) // 1500) % 331]
    return records(pos.astype(np.float32))


@pytest.mark.parametrize("kind", ["clump", "two", "ramp"])
@pytest.mark.parametrize("digit_bits", [8, 11])
@pytest.mark.parametrize("bits", [30, 63])
def test_sort_skewed_digits_give_the_oracle_tree(kind, digit_bits, bits):
    """The onesweep ranking, look-back and scatter under heavy digit skew
    (lane masks of whole warps on one digit, runs of equal keys across tile
    borders, a partial last tile): codes, ids and every node word equal the
    oracle's stable sort and tree."""
    tris = _skewed_scene(kind, 100_003, seed={"clump": 1, "two": 2, "ramp": 3}[kind])
    lb = O.lbvh_build(tris, bits)
    ctor = P.lbvh_constructor(morton_bits=bits, digit_bits=digit_bits)
    bvh = ctor.build(P.cuda_ftl(tris))
    codes = lb.codes if bits == 63 else lb.codes.astype(np.uint32)
    assert_build_equals(bvh, codes, lb.ids, lb.nodes)


@pytest.mark.parametrize("kind", ["clump", "ramp"])
@pytest.mark.parametrize("mode", ["cis", "dis", "shadow_cis"])
def test_trace_through_collapsed_leaves_of_many_triangles(kind, mode):
    """Leaves collapsed from equal codes hold up to ~100,000 triangles here,
    far past the 64 a link's count field holds, so the traversal reads their
    count from the triangle record: rays aimed at the clumps (and some that
    miss) give the oracle's hits and per-ray counts."""
    tris = _skewed_scene(kind, 100_003, seed={"clump": 1, "ramp": 3}[kind])
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    rng = np.random.default_rng(11)
    pos = np.asarray(tris[:, :9], np.float32).reshape(-1, 3, 3)
    tgt = pos[rng.integers(0, pos.shape[0], 1024)].mean(axis=1)
    o = (tgt + rng.normal(0, 2.0, (1024, 3))).astype(np.float32)
    d = (tgt - o + rng.normal(0, 0.05, (1024, 3))).astype(np.float32)
    m = np.full(1024, S.FLT_MAX, np.float32)
    ref, st_ref, overflow = O.trace(lb.nodes, srt, o, d, m, ORC[mode], 64, stats=True)
    assert not overflow
    bvh = gpu_build(tris, 30)
    got, st = gpu_trace(bvh, o, d, m, MODES[mode], stats=True)
    assert_hits_equal(got, ref)
    np.testing.assert_array_equal(st, st_ref)
    assert (got["t"] != np.float32(S.FLT_MAX)).mean() > 0.2


def test_rebuild_reuses_buffers_and_matches():
    """Rebuilding with a second, smaller scene through the same constructor
    (the -R path, rta/main.cpp:389-400) gives that scene's tree."""
    ctor = P.lbvh_constructor(morton_bits=30)
    big = S.terrain(128, 64, seed=4)
    small = S.clusters(4, 1000, seed=6)
    ctor.build(P.cuda_ftl(big))
    bvh = ctor.build(P.cuda_ftl(small))
    lb = O.lbvh_build(small, 30)
    assert_build_equals(bvh, lb.codes.astype(np.uint32), lb.ids, lb.nodes)


# --------------------------------------------------------------------------- #
# rays and traversal                                                           #
# --------------------------------------------------------------------------- #

def test_camera_kernel_matches_reference_golden(golden_dir):
    z = np.load(os.path.join(golden_dir, "sphere_trace.npz"))
    g = P.cam_ray_generator_shirley(int(z["w"]), int(z["h"]))
    g.setup(z["cam_pos"], z["cam_dir"], z["cam_up"], 60.0)
    import ctypes as C
    L.check(L.load().rta_setup_shirley_rays(
        P._ptr(g.gpu_direction), P._ptr(g.gpu_origin), P._ptr(g.gpu_maxt), float(z["tan_half"]),
        float(g.aspect), g.w, g.h, (C.c_float * 3)(*z["cam_dir"].tolist()),
        (C.c_float * 3)(*z["cam_pos"].tolist()), (C.c_float * 3)(*z["cam_up"].tolist()),
        S.FLT_MAX, P._stream()), "rta_setup_shirley_rays")
    torch.cuda.synchronize()
    rays = np.concatenate([g.gpu_origin.cpu().numpy().reshape(-1, 3),
                           g.gpu_direction.cpu().numpy().reshape(-1, 3),
                           g.gpu_maxt.cpu().numpy()[:, None]], axis=1)
    assert sha(rays.astype(np.float32)) == str(z["rays_sha"])


@pytest.mark.parametrize("mode", list(MODES))
def test_trace_matches_reference_golden(golden_dir, mode):
    z = np.load(os.path.join(golden_dir, "sphere_trace.npz"))
    tris = records(z["pos"])
    bvh = gpu_build(tris)
    o, d, m = O.shirley_rays(z["tan_half"], np.float32(np.float32(z["w"]) / np.float32(z["h"])),
                             int(z["w"]), int(z["h"]), z["cam_dir"], z["cam_pos"], z["cam_up"])
    hits = gpu_trace(bvh, o, d, m, MODES[mode])
    if mode == "cis":
        assert_hits_equal(hits, z["cis_hits"])
    assert sha(hits) == str(z[f"{mode}_sha"])


def test_trace_matches_cpu_plugin_golden(golden_dir):
    """Config 1: hits by original triangle id equal the reference CPU plugin's."""
    z = np.load(os.path.join(golden_dir, "sphere_trace.npz"))
    bvh = gpu_build(records(z["pos"]))
    o, d, m = O.shirley_rays(z["tan_half"], np.float32(np.float32(z["w"]) / np.float32(z["h"])),
                             int(z["w"]), int(z["h"]), z["cam_dir"], z["cam_pos"], z["cam_up"])
    hits = gpu_trace(bvh, o, d, m, L.TRACE_CIS)
    valid = hits["t"] != np.float32(S.FLT_MAX)
    ids = np.where(valid, bvh.index_buffer[hits["ref"]], np.uint32(0xFFFFFFFF))
    np.testing.assert_array_equal(ids, z["bbvh_id"])
    np.testing.assert_array_equal(hits["t"].view(np.uint32), z["bbvh_t"].view(np.uint32))


@pytest.mark.parametrize("mode", ["cis", "dis"])
def test_terrain_trace_matches_reference_golden(golden_dir, mode):
    z = np.load(os.path.join(golden_dir, "terrain_trace.npz"))
    bvh = gpu_build(records(z["pos"]))
    o, d, m = O.shirley_rays(z["tan_half"], np.float32(np.float32(z["w"]) / np.float32(z["h"])),
                             int(z["w"]), int(z["h"]), z["cam_dir"], z["cam_pos"], z["cam_up"])
    hits = gpu_trace(bvh, o, d, m, MODES[mode])
    assert sha(hits) == sha(z[f"{mode}_hits"])


@pytest.mark.parametrize("mode", list(MODES))
def test_trace_matches_oracle_terrain(mode):
    tris = S.terrain(256, 128, seed=7)
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=480, h=270)
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    ref, _, _ = O.trace(lb.nodes, srt, o, d, m, ORC[mode], 64)
    bvh = gpu_build(tris)
    assert_hits_equal(gpu_trace(bvh, o, d, m, MODES[mode]), ref)


@pytest.mark.parametrize("bits", [30, 63])
@pytest.mark.parametrize("mode", ["cis", "dis", "shadow_cis"])
def test_trace_matches_oracle_incoherent(bits, mode):
    tris = S.clusters(64, 1024, seed=9)
    lb = O.lbvh_build(tris, bits)
    srt = O.permute(tris, lb.ids)
    o, d, m = S.incoherent_rays(200_000, seed=9)
    ref, st_ref, _ = O.trace(lb.nodes, srt, o, d, m, ORC[mode], 256, stats=True)
    bvh = gpu_build(tris, bits)
    hits, st = gpu_trace(bvh, o, d, m, MODES[mode], stats=True)
    assert_hits_equal(hits, ref)
    np.testing.assert_array_equal(st, st_ref)   # same visiting order, node for node
    assert bvh.status() & L.DEV_STACK_OVERFLOW == 0


def test_miss_keeps_record_fields():
    """A miss writes only t (kernels.cu:794-796 reads the record first)."""
    tris = S.terrain(8, 8)
    bvh = gpu_build(tris)
    o = np.array([0, 5, 0], np.float32)
    d = np.array([0, 1, 0], np.float32)
    init = np.zeros(1, O.HIT_DTYPE)
    init["t"], init["beta"], init["gamma"], init["ref"] = 3.0, 0.25, 0.5, 77
    h = gpu_trace(bvh, o, d, np.array([S.FLT_MAX], np.float32), L.TRACE_CIS, hits_init=init)
    assert h["t"][0] == np.float32(S.FLT_MAX)
    assert (h["beta"][0], h["gamma"][0], h["ref"][0]) == (np.float32(0.25), np.float32(0.5), 77)


def test_max_t_is_honoured():
    tris = S.terrain(64, 32, seed=1)
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=160, h=90)
    o, d, _ = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    m = np.full(cam.w * cam.h, 1.7, np.float32)
    ref, _, _ = O.trace(lb.nodes, srt, o, d, m, O.CIS, 64)
    got = gpu_trace(gpu_build(tris), o, d, m, L.TRACE_CIS)
    assert_hits_equal(got, ref)
    assert (got["t"][got["t"] < 3e38] <= 1.7).all()


# --------------------------------------------------------------------------- #
# frame: primary + one diffuse bounce                                          #
# --------------------------------------------------------------------------- #

def test_frame_bounce_matches_oracle():
    tris = S.terrain(128, 64, seed=5)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=320, h=180)
    s = P.create_rt_set(tris, cam.w, cam.h)
    s.rgen.setup(cam.pos, cam.dir, cam.up, cam.fovy)
    b = P.diffuse_bounce_collector(cam.w, cam.h, seed=13, eps=1e-4)
    s.rt.ray_generator(s.rgen)
    s.rt.ray_bouncer(b)
    s.rt.trace()
    assert len(s.rt.timings) == 2
    torch.cuda.synchronize()
    prim = b.intersections()
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    ref, _, _ = O.trace(lb.nodes, srt, o, d, m, O.CIS, 64)
    assert_hits_equal(prim, ref)
    bo, bd, bm, bsrc = O.diffuse_bounce(srt, o, d, ref, seed=13, eps=1e-4)
    cnt = b.bounce_count()
    assert cnt == bm.shape[0] and cnt > 0
    f = b.frame
    got_o = P.device_view(f.orig, 3 * cnt).cpu().numpy()
    got_d = P.device_view(f.dir, 3 * cnt).cpu().numpy()
    got_src = P.device_view(f.src, cnt, "<u4").cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(got_src, bsrc)
    np.testing.assert_array_equal(got_o.view(np.uint32), bo.view(np.uint32))
    np.testing.assert_array_equal(got_d.view(np.uint32), bd.view(np.uint32))
    bref, _, _ = O.trace(lb.nodes, srt, bo, bd, bm, O.CIS, 64)
    got_h = P.device_view(f.hits, 4 * cnt).cpu().numpy().view(O.HIT_DTYPE)
    assert_hits_equal(got_h, bref)


def test_frame_on_pinned_host_buffers_matches_oracle():
    """rta_frame_run with the rays and primary hits in pinned host memory
    (read and written by the kernels directly) gives the oracle's hits and
    bounce rays, as the device-resident frame does."""
    import ctypes as C
    tris = S.terrain(128, 64, seed=5)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=320, h=180)
    n = cam.w * cam.h
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    ho = torch.from_numpy(np.ascontiguousarray(o, np.float32).reshape(-1)).pin_memory()
    hd = torch.from_numpy(np.ascontiguousarray(d, np.float32).reshape(-1)).pin_memory()
    hm = torch.from_numpy(np.ascontiguousarray(m, np.float32).reshape(-1)).pin_memory()
    hh = torch.zeros(4 * n, dtype=torch.float32).pin_memory()
    bvh = gpu_build(tris, 30)
    lib = L.load()
    fh = C.c_void_p()
    L.check(lib.rta_frame_create(C.byref(fh), n), "rta_frame_create")
    try:
        f = L.FrameView()
        L.check(lib.rta_frame_get(fh, C.byref(f)), "rta_frame_get")
        L.check(lib.rta_frame_run(fh, C.byref(bvh.view), P._ptr(ho), P._ptr(hd), P._ptr(hm), n, P._ptr(hh),
                                  L.TRACE_CIS, 13, np.float32(1e-4), P._stream()), "rta_frame_run")
        torch.cuda.synchronize()
        lb = O.lbvh_build(tris, 30)
        srt = O.permute(tris, lb.ids)
        ref, _, _ = O.trace(lb.nodes, srt, o, d, m, O.CIS, 64)
        assert_hits_equal(hh.numpy().view(O.HIT_DTYPE), ref)
        bo, bd, bm, bsrc = O.diffuse_bounce(srt, o, d, ref, seed=13, eps=1e-4)
        cnt = int(P.device_view(f.count, 1, "<u4").cpu().numpy().view(np.uint32)[0])
        assert cnt == bm.shape[0] and cnt > 0
        got_o = P.device_view(f.orig, 3 * cnt).cpu().numpy()
        np.testing.assert_array_equal(got_o.view(np.uint32), bo.view(np.uint32))
        bref, _, _ = O.trace(lb.nodes, srt, bo, bd, bm, O.CIS, 64)
        assert_hits_equal(P.device_view(f.hits, 4 * cnt).cpu().numpy().view(O.HIT_DTYPE), bref)
    finally:
        lib.rta_frame_destroy(fh)


def test_rebinding_contract():
    """rt.acceleration_structure(new_as) makes the tracer use the new tree
    (bbvh-cuda.h:89-92, rta/main.cpp:389-400)."""
    a = S.terrain(32, 16, seed=1)
    b = S.clusters(4, 256, seed=2)
    s = P.create_rt_set(a, 64, 64)
    new_as = s.ctor.build(P.cuda_ftl(b))
    s.rt.acceleration_structure(new_as)
    assert s.rt.acceleration_structure() is new_as and s.rt.bbvh is new_as


# --------------------------------------------------------------------------- #
# full configuration-2 size                                                    #
# --------------------------------------------------------------------------- #

class _FullTerrain:
    """The benchmarked configuration: the 1,048,576-triangle terrain (seed
    0), its 1920x1080 camera frame and one diffuse bounce per hit (seed 0,
    eps 1e-4), all computed by the oracle once per module."""

    def __init__(self):
        self.tris = S.terrain(1024, 512, seed=0)
        self.lb = O.lbvh_build(self.tris, 30)
        self.srt = O.permute(self.tris, self.lb.ids)
        cam = S.terrain_camera()
        self.cam = cam
        self.o, self.d, self.m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
        self.ref, _, _ = O.trace(self.lb.nodes, self.srt, self.o, self.d, self.m, O.CIS, 64)
        self.bo, self.bd, self.bm, self.bsrc = O.diffuse_bounce(self.srt, self.o, self.d, self.ref, seed=0,
                                                                eps=1e-4)
        self.bref, _, _ = O.trace(self.lb.nodes, self.srt, self.bo, self.bd, self.bm, O.CIS, 64)


@pytest.fixture(scope="module")
def full_terrain():
    return _FullTerrain()


def test_full_size_terrain_build_and_frame(full_terrain):
    """1,048,576-triangle terrain and the 1920x1080 frame: the whole tree is
    bit-identical to the oracle's, and so is every primary hit."""
    ft = full_terrain
    bvh = gpu_build(ft.tris, 30)
    codes = bvh.codes()
    assert (np.diff(codes.astype(np.int64)) >= 0).all()
    ids = bvh.index_buffer
    assert np.array_equal(np.sort(ids), np.arange(ft.tris.shape[0], dtype=np.uint32))
    assert_build_equals(bvh, ft.lb.codes.astype(np.uint32), ft.lb.ids, ft.lb.nodes)
    assert_hits_equal(gpu_trace(bvh, ft.o, ft.d, ft.m, L.TRACE_CIS), ft.ref)


def _device(a, dtype=np.float32):
    return torch.from_numpy(np.ascontiguousarray(a, dtype).reshape(-1).copy()).to("cuda")


def test_full_size_fused_frame_matches_oracle(full_terrain):
    """The benchmarked frame exactly as bench.py times it: rta_frame_run (the
    fused primary + bounce trace launch and the bounce gather) on the
    1,048,576-triangle terrain at 1920x1080, seed 0, eps 1e-4.  Every primary
    hit, the bounce count, every bounce ray (origin, direction, max_t, source
    pixel) and every bounce hit equal the oracle's, bit for bit."""
    import ctypes as C
    ft = full_terrain
    bvh = gpu_build(ft.tris, 30)
    n = ft.m.shape[0]
    o, d, m = _device(ft.o), _device(ft.d), _device(ft.m)
    hits = torch.empty(4 * n, dtype=torch.float32, device="cuda")
    lib = L.load()
    fh = C.c_void_p()
    L.check(lib.rta_frame_create(C.byref(fh), n), "rta_frame_create")
    try:
        f = L.FrameView()
        L.check(lib.rta_frame_get(fh, C.byref(f)), "rta_frame_get")
        for _ in range(2):   # the second run reuses the frame's buffers and counters
            hits.fill_(0)
            L.check(lib.rta_frame_run(fh, C.byref(bvh.view), P._ptr(o), P._ptr(d), P._ptr(m), n, P._ptr(hits),
                                      L.TRACE_CIS, 0, np.float32(1e-4), P._stream()), "rta_frame_run")
            flags = C.c_uint32(0)
            L.check(lib.rta_frame_status(fh, P._stream(), C.byref(flags)), "rta_frame_status")
            assert flags.value == 0
            assert_hits_equal(hits.cpu().numpy().view(O.HIT_DTYPE), ft.ref)
            cnt = int(P.device_view(f.count, 1, "<u4").cpu().numpy().view(np.uint32)[0])
            assert cnt == ft.bm.shape[0] > 700000
            np.testing.assert_array_equal(P.device_view(f.src, cnt, "<u4").cpu().numpy().view(np.uint32), ft.bsrc)
            np.testing.assert_array_equal(P.device_view(f.orig, 3 * cnt).cpu().numpy().view(np.uint32),
                                          ft.bo.reshape(-1).view(np.uint32))
            np.testing.assert_array_equal(P.device_view(f.dir, 3 * cnt).cpu().numpy().view(np.uint32),
                                          ft.bd.reshape(-1).view(np.uint32))
            np.testing.assert_array_equal(P.device_view(f.maxt, cnt).cpu().numpy().view(np.uint32),
                                          ft.bm.view(np.uint32))
            assert_hits_equal(P.device_view(f.hits, 4 * cnt).cpu().numpy().view(O.HIT_DTYPE), ft.bref)
    finally:
        lib.rta_frame_destroy(fh)


def test_full_size_host_frames_match_oracle(full_terrain):
    """The e2e path of the bench, rta_host_frames_run on pinned host buffers,
    at full size.  The tree is rebuilt on a side stream behind a delay and
    the frames are queued on that stream with no host synchronisation: the
    frames' own streams must wait for the rebuild (rta_lbvh::ready), so the
    hits are the new tree's.  Three frames in a row use both buffer sets."""
    ft = full_terrain
    n = ft.m.shape[0]
    ctor = P.lbvh_constructor(morton_bits=30)
    # another tree of the same size first, so the rebuild reuses the buffers
    # (a reallocation would synchronise the device and hide the ordering)
    ctor.build(P.cuda_ftl(S.terrain(1024, 512, seed=7)))
    torch.cuda.synchronize()
    ho = torch.from_numpy(np.ascontiguousarray(ft.o, np.float32).reshape(-1)).pin_memory()
    hd = torch.from_numpy(np.ascontiguousarray(ft.d, np.float32).reshape(-1)).pin_memory()
    hm = torch.from_numpy(np.ascontiguousarray(ft.m, np.float32).reshape(-1)).pin_memory()
    outs = [(torch.zeros(4 * n, dtype=torch.float32).pin_memory(),
             torch.zeros(4 * n, dtype=torch.float32).pin_memory(),
             torch.zeros(1, dtype=torch.int32).pin_memory()) for _ in range(3)]
    tri_dev = P.cuda_ftl(ft.tris)
    hf = P.host_frames(n)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())   # the triangle upload
    with torch.cuda.stream(side):
        torch.cuda._sleep(200_000_000)   # about 0.1 s of GPU time before the rebuild starts
        bvh = ctor.build(tri_dev)
        for h_hits, h_bhits, h_cnt in outs:
            hf.run(bvh, ho, hd, hm, h_hits, h_bhits, h_cnt, L.TRACE_CIS, 0, 1e-4, n)
    side.synchronize()
    nb = ft.bm.shape[0]
    for h_hits, h_bhits, h_cnt in outs:
        assert int(h_cnt.item()) == nb
        assert_hits_equal(h_hits.numpy().view(O.HIT_DTYPE), ft.ref)
        assert_hits_equal(h_bhits.numpy().view(O.HIT_DTYPE)[:nb], ft.bref)


def test_full_size_incoherent_clusters_build_and_trace():
    """The 4,194,304-triangle cluster soup with 63-bit codes and 8,388,608
    incoherent rays: tree and every hit bit-identical to the oracle's, and
    the closest-hit trace of a quarter of the rays in the DIS order too."""
    tris = S.clusters(256, 16384, seed=0)
    lb = O.lbvh_build(tris, 63)
    bvh = gpu_build(tris, 63)
    assert (np.diff(bvh.codes().astype(np.float64)) >= 0).all()
    assert_build_equals(bvh, lb.codes, lb.ids, lb.nodes)
    o, d, m = S.incoherent_rays(1 << 23, seed=0)
    srt = O.permute(tris, lb.ids)
    ref, st_ref, overflow = O.trace(lb.nodes, srt, o, d, m, O.CIS, 128, stats=True)
    assert not overflow
    got, st = gpu_trace(bvh, o, d, m, L.TRACE_CIS, stats=True)
    assert_hits_equal(got, ref)
    np.testing.assert_array_equal(st, st_ref)   # same nodes and triangles visited per ray
    q = slice(0, 1 << 21)
    ref_dis, _, _ = O.trace(lb.nodes, srt, o.reshape(-1, 3)[q], d.reshape(-1, 3)[q], m[q], O.DIS, 128)
    assert_hits_equal(gpu_trace(bvh, o.reshape(-1, 3)[q], d.reshape(-1, 3)[q], m[q], L.TRACE_DIS), ref_dis)
    assert bvh.status() & (L.DEV_STACK_OVERFLOW | L.DEV_ITER_LIMIT | L.DEV_BAD_LINK | L.DEV_SPIN_TIMEOUT) == 0


# --------------------------------------------------------------------------- #
# host shading on the device                                                  #
# --------------------------------------------------------------------------- #

def gpu_shade(hits, tris, w, h, lights, binary, bg):
    import ctypes as C
    dev = torch.device("cuda")
    hd = torch.from_numpy(np.ascontiguousarray(hits).view(np.float32).reshape(-1).copy()).to(dev)
    td = torch.from_numpy(np.ascontiguousarray(tris, np.float32).reshape(-1).copy()).to(dev)
    img = torch.zeros(w * h * 3, dtype=torch.uint8, device=dev)
    lt = np.ascontiguousarray(lights, np.float32)
    bgv = np.ascontiguousarray(bg, np.float32)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    L.check(L.load().rta_shade_lambert(P._ptr(hd), P._ptr(td), tris.shape[0], w, h,
                                       lt.ctypes.data_as(C.c_void_p), lt.shape[0], int(binary),
                                       bgv.ctypes.data_as(C.c_void_p), P._ptr(img), P._ptr(flags),
                                       P._stream()), "rta_shade_lambert")
    torch.cuda.synchronize()
    assert int(flags.item()) == 0
    return img.cpu().numpy().reshape(h, w, 3)


def test_shading_matches_reference_golden(golden_dir):
    z = np.load(os.path.join(golden_dir, "shade_sphere.npz"))
    sp = np.load(os.path.join(golden_dir, "sphere_trace.npz"))
    w, h = int(sp["w"]), int(sp["h"])
    hits = sp["cis_hits"].view(O.HIT_DTYPE)
    np.testing.assert_array_equal(gpu_shade(hits, z["tris"], w, h, z["lights"], False, z["bg"]), z["image"])
    np.testing.assert_array_equal(gpu_shade(hits, z["tris"], w, h, z["lights"], True, z["bg"]), z["binary"])


def test_direct_diffuse_illumination_full_frame_matches_oracle(tmp_path):
    """The terrain's 1920x1080 primary frame shaded on the device through the
    plugin mirror (trace, then shade) equals the oracle's host shading."""
    tris = S.terrain(1024, 512, seed=0)
    s = P.create_rt_set(tris, 1920, 1080)
    cam = S.terrain_camera()
    s.rgen.setup(cam.pos, cam.dir, cam.up, cam.fovy)
    shader = P.direct_diffuse_illumination(1920, 1080)
    s.rt.ray_generator(s.rgen)
    s.rt.ray_bouncer(shader)
    s.rt.trace()
    shader.triangle_ptr(s.as_.triangle_data)
    lights = [((1.5, 2.0, 1.0), (0.8, 0.75, 0.7)), ((-1.0, 1.0, -0.5), (0.2, 0.25, 0.35))]
    shader.reset((0.05, 0.1, 0.2))
    for at, col in lights:
        shader.add_pointlight(at, col)
    shader.shade()
    got = shader.pixels()
    hits = shader.intersections()
    want = O.shade_lambert(s.as_.canonical_triangle_ptr(), hits, 1920, 1080,
                           np.array([list(a) + list(c) for a, c in lights], np.float32), False, (0.05, 0.1, 0.2))
    np.testing.assert_array_equal(got, want)
    path = str(tmp_path / "frame.png")
    shader.save(path)
    assert os.path.getsize(path) > 1000


def test_host_frames_pipeline_matches_device_frames():
    """Three frames in a row through rta_host_frames_run (pinned host
    buffers, two frames in flight) equal rta_frame_run on device buffers,
    primary and bounce hits and bounce counts, each frame with its own seed
    and its own output buffers."""
    import ctypes as C
    tris = S.terrain(128, 64, seed=5)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=320, h=180)
    n = cam.w * cam.h
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    ho = torch.from_numpy(np.ascontiguousarray(o, np.float32).reshape(-1)).pin_memory()
    hd = torch.from_numpy(np.ascontiguousarray(d, np.float32).reshape(-1)).pin_memory()
    hm = torch.from_numpy(np.ascontiguousarray(m, np.float32).reshape(-1)).pin_memory()
    bvh = gpu_build(tris, 30)
    hf = P.host_frames(n)
    outs = []
    for seed in (3, 4, 5):
        hh = torch.zeros(4 * n, dtype=torch.float32).pin_memory()
        hb = torch.zeros(4 * n, dtype=torch.float32).pin_memory()
        hc = torch.zeros(1, dtype=torch.int32).pin_memory()
        hf.run(bvh, ho, hd, hm, hh, hb, hc, L.TRACE_CIS, seed, 1e-4)
        outs.append((seed, hh, hb, hc))
    torch.cuda.current_stream().synchronize()
    lib = L.load()
    dev = torch.device("cuda")
    do, dd, dm = ho.to(dev), hd.to(dev), hm.to(dev)
    for seed, hh, hb, hc in outs:
        fh = C.c_void_p()
        L.check(lib.rta_frame_create(C.byref(fh), n), "rta_frame_create")
        f = L.FrameView()
        L.check(lib.rta_frame_get(fh, C.byref(f)), "rta_frame_get")
        dh = torch.zeros(4 * n, dtype=torch.float32, device=dev)
        L.check(lib.rta_frame_run(fh, C.byref(bvh.view), P._ptr(do), P._ptr(dd), P._ptr(dm), n, P._ptr(dh),
                                  L.TRACE_CIS, seed, np.float32(1e-4), P._stream()), "rta_frame_run")
        torch.cuda.synchronize()
        cnt = int(P.device_view(f.count, 1, "<u4").cpu().numpy().view(np.uint32)[0])
        assert int(hc.item()) == cnt > 0
        assert_hits_equal(hh.numpy().view(O.HIT_DTYPE), dh.cpu().numpy().view(O.HIT_DTYPE))
        want_b = P.device_view(f.hits, 4 * cnt).cpu().numpy().view(O.HIT_DTYPE)
        got_b = hb.numpy().view(O.HIT_DTYPE)[:cnt]
        np.testing.assert_array_equal(got_b["t"].view(np.uint32), want_b["t"].view(np.uint32))
        v = got_b["t"] != np.float32(S.FLT_MAX)
        for fld in ("beta", "gamma", "ref"):
            np.testing.assert_array_equal(got_b[fld][v].view(np.uint32), want_b[fld][v].view(np.uint32))
        lib.rta_frame_destroy(fh)


def test_frame_trace_timing():
    """rta_frame_set_timing / rta_frame_trace_ms: invalid before a timed run,
    then the trace time of the last frame, below the whole frame's time."""
    import ctypes as C
    tris = S.terrain(128, 64, seed=5)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=320, h=180)
    n = cam.w * cam.h
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    dev = torch.device("cuda")
    do, dd, dm = (torch.from_numpy(np.ascontiguousarray(x, np.float32).reshape(-1)).to(dev) for x in (o, d, m))
    hh = torch.zeros(4 * n, dtype=torch.float32, device=dev)
    bvh = gpu_build(tris, 30)
    lib = L.load()
    fh = C.c_void_p()
    L.check(lib.rta_frame_create(C.byref(fh), n), "rta_frame_create")
    try:
        ms = C.c_float(0)
        assert lib.rta_frame_trace_ms(fh, C.byref(ms)) == L.ERR_INVALID
        L.check(lib.rta_frame_set_timing(fh, 1), "rta_frame_set_timing")
        for mode in (L.TRACE_CIS, L.TRACE_DIS):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            L.check(lib.rta_frame_run(fh, C.byref(bvh.view), P._ptr(do), P._ptr(dd), P._ptr(dm), n, P._ptr(hh),
                                      mode, 3, np.float32(1e-4), P._stream()), "rta_frame_run")
            e1.record()
            e1.synchronize()
            L.check(lib.rta_frame_trace_ms(fh, C.byref(ms)), "rta_frame_trace_ms")
            assert 0.0 < ms.value <= e0.elapsed_time(e1) * 1.05 + 0.01
    finally:
        lib.rta_frame_destroy(fh)
