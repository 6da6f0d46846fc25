"""The drop-in itself: the rta plugin bbvh-gb300.so (plugin/bbvh_gb300.cpp)
loaded by a headless rta driver (plugin/rta_harness.cpp) and driven through
rta's interfaces in the driver's order: initialize, parse_cmdline,
create_rt_set, ray_bouncer / ray_generator, setup + trace, and a -R rebuild
through the constructor with the acceleration_structure() re-binding
(rta/main.cpp:382-405, 479-488).  The hits equal the reference's own
kernels' (golden digests) and the oracle's, bit for bit.

The plugin compiles against the reference's librta headers, which the
plugin Makefile stages into plugin/_build/gen; where they were never staged
the tests are skipped with that reason."""
import ctypes as C
import hashlib
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402
from rta_gb300 import scenes as S  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLUGIN_DIR = os.path.join(ROOT, "plugin")
BUILD = os.path.join(PLUGIN_DIR, "_build")
PLUGIN = os.path.join(BUILD, "bbvh-gb300.so")
HARNESS = os.path.join(BUILD, "rta_harness")
HARNESS_LIB = os.path.join(BUILD, "librta_harness.so")
STAGED = os.path.join(BUILD, "gen", "librta", "librta.h")


@pytest.fixture(scope="module")
def plugin():
    if not os.path.exists(STAGED):
        pytest.skip("the reference's librta headers were never staged into plugin/_build/gen")
    subprocess.run(["make", "-s", "-C", PLUGIN_DIR], check=True)
    return PLUGIN


def write_scene(path, tris, cam):
    hdr = np.array([tris.shape[0], cam.w, cam.h], np.uint32)
    camv = np.concatenate([[np.float32(cam.fovy)], cam.pos, cam.dir, cam.up]).astype(np.float32)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(camv.tobytes())
        f.write(np.ascontiguousarray(tris, np.float32).tobytes())


def run_harness(tmp_path, scenes, args):
    paths = []
    for k, (tris, cam) in enumerate(scenes):
        p = str(tmp_path / f"scene{k}.bin")
        write_scene(p, tris, cam)
        paths.append(p)
    prefix = str(tmp_path / "frame")
    r = subprocess.run([HARNESS, PLUGIN, prefix, *paths, "--", *args], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = []
    for k in range(len(scenes)):
        hits = np.fromfile(f"{prefix}.{k}.hits", dtype=O.HIT_DTYPE)
        ids = np.fromfile(f"{prefix}.{k}.ids", dtype=np.uint32)
        out.append((hits, ids))
    with open(prefix + ".log") as f:
        log = f.read()
    return out, log, r.stdout, prefix


def sphere_scene():
    z = np.load(os.path.join(ROOT, "tests", "golden", "sphere_trace.npz"))
    p = np.asarray(z["pos"], np.float32).reshape(-1, 3, 3)
    tris = S._records(p[:, 0], p[:, 1], p[:, 2])
    cam = S.Camera(z["cam_pos"], z["cam_pos"] + z["cam_dir"], z["cam_up"], fovy=60.0, w=int(z["w"]), h=int(z["h"]))
    cam.dir = np.asarray(z["cam_dir"], np.float32)
    return tris, cam, z


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_frame(tris, cam, mode):
    lb = O.lbvh_build(tris, 30)
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    hits, _, _ = O.trace(lb.nodes, O.permute(tris, lb.ids), o, d, m, mode, 64)
    return hits, lb.ids


def assert_same_hits(a, b):
    np.testing.assert_array_equal(a.view(np.uint32).reshape(-1, 4)[:, :3], b.view(np.uint32).reshape(-1, 4)[:, :3])
    valid = a["t"] != np.float32(S.FLT_MAX)
    np.testing.assert_array_equal(a["ref"][valid], b["ref"][valid])


@pytest.mark.parametrize("args,golden", [(["-t", "cis"], "cis_sha"), (["-t", "dis", "-s"], "shadow_dis_sha"),
                                         (["-A"], "cis_aila_sha")])
def test_plugin_frame_and_rebuild_match_reference(plugin, tmp_path, args, golden):
    """Frame 0: the 6,240-triangle sphere view through create_rt_set; every
    hit record equals the reference kernels' (golden digest).  Frame 1: a -R
    rebuild with another scene (a 4,096-triangle terrain) re-bound to the
    tracer; every hit equals the oracle's for that scene."""
    tris0, cam0, z = sphere_scene()
    tris1 = S.terrain(64, 32, seed=1)
    cam1 = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=cam0.w, h=cam0.h)
    frames, log, _, _ = run_harness(tmp_path, [(tris0, cam0), (tris1, cam1)], args)
    (h0, ids0), (h1, ids1) = frames
    assert sha(h0) == str(z[golden])
    mode = {"cis_sha": O.CIS, "shadow_dis_sha": O.DIS | O.SHADOW, "cis_aila_sha": O.CIS | O.AILA}[golden]
    want1, lb_ids1 = oracle_frame(tris1, cam1, mode)
    assert_same_hits(h1, want1)
    np.testing.assert_array_equal(ids1, lb_ids1)   # canonical triangles = input records in Morton order
    np.testing.assert_array_equal(ids0, O.lbvh_build(tris0, 30).ids)
    assert log.count("frame ") == 2 and "passes 1 " in log


def test_plugin_verbose_prints_the_build_passes(plugin, tmp_path):
    """-v prints each build pass's time, as lbvh_constructor::buildCUDA does
    (lbvh.h:172-204), and 63-bit codes give the oracle's hits."""
    tris, cam = S.clusters(8, 512, seed=2), S.Camera((0.0, 0.0, 14.0), (0.0, 0.0, 0.0), w=96, h=64)
    frames, _, stdout, _ = run_harness(tmp_path, [(tris, cam)], ["-v", "--morton-bits", "63"])
    for line in ("Time for calculating Morton Codes:", "Time for sorting Morton Codes:",
                 "Time for tree construction:", "BVH finished. Total time:"):
        assert line in stdout, stdout
    lb = O.lbvh_build(tris, 63)
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    want, _, _ = O.trace(lb.nodes, O.permute(tris, lb.ids), o, d, m, O.CIS, 128)
    assert_same_hits(frames[0][0], want)


def test_plugin_loads_in_process(plugin):
    """The plugin resolves librta's symbols from a driver loaded first with
    RTLD_GLOBAL, as rta/main.cpp loads plugins; initialize() announces CUDA."""
    host = C.CDLL(HARNESS_LIB, mode=C.RTLD_GLOBAL)
    lib = C.CDLL(PLUGIN)
    lib.description.restype = C.c_char_p
    assert b"sm_103a" in lib.description()
    lib.initialize()
    assert host is not None


def test_plugin_mamo_dumps(plugin, tmp_path):
    """The plugin's tree, triangle and ray dumps (as rta -m writes them) are
    the reference dump format (checked byte for byte against the reference's
    own dump code in tests/test_dumps.py) of the oracle's tree, Morton-ordered
    triangles and camera rays."""
    from rta_gb300 import plugin as P
    tris = S.terrain(32, 16, seed=4)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=64, h=36)
    _, _, _, prefix = run_harness(tmp_path, [(tris, cam)], ["-t", "cis"])
    lb = O.lbvh_build(tris, 30)
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    with open(prefix + ".0.bvh") as f:
        assert f.read() == P.format_bvh_dump(lb.nodes)
    with open(prefix + ".0.tri") as f:
        assert f.read() == P.format_tri_dump(O.permute(tris, lb.ids))
    with open(prefix + ".0.ray") as f:
        assert f.read() == P.format_ray_dump(o, d, m, cam.w, cam.h)
