"""Pins the CPU oracle to golden data produced by the reference's own code
(tests/golden/make_golden.py): the LBVH kernels of bbvh-cuda/lbvh-kernels.cu,
the 2F4 trace kernels of bbvh-cuda/kernels.cu, the camera kernel of
librta/cuda-kernels.cu and the CPU plugin bbvh.so."""
import hashlib
import os

import numpy as np
import pytest

from oracle import oracle as O
from rta_gb300 import scenes as S

MODES = {"cis": O.CIS, "dis": O.DIS, "shadow_cis": O.CIS | O.SHADOW,
         "shadow_dis": O.DIS | O.SHADOW, "cis_aila": O.CIS | O.AILA, "dis_aila": O.DIS | O.AILA}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def records(pos):
    p = np.asarray(pos, np.float32).reshape(-1, 3, 3)
    return S._records(p[:, 0], p[:, 1], p[:, 2])


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def case_names(golden_dir):
    z = load(golden_dir, "lbvh_cases.npz")
    return sorted({k.split("/")[0] for k in z.files})


@pytest.mark.parametrize("case", ["n1", "n2", "n3", "n7", "dup64", "rand100", "clump",
                                  "terrain16x8", "clusters4x64", "sphere"])
def test_lbvh_matches_reference(golden_dir, case):
    z = load(golden_dir, "lbvh_cases.npz")
    tris = records(z[f"{case}/pos"])
    lb = O.lbvh_build(tris, 30)
    assert lb.flags & O.FLAG_CODE0_RACE == 0
    np.testing.assert_array_equal(lb.codes.astype(np.uint32), z[f"{case}/codes"])
    np.testing.assert_array_equal(lb.ids, z[f"{case}/ids"])
    np.testing.assert_array_equal(lb.scene, z[f"{case}/scene"])
    np.testing.assert_array_equal(lb.nodes.view(np.uint32), z[f"{case}/nodes"].view(np.uint32))


def test_golden_has_collapsed_leaves(golden_dir):
    """The duplicate cases exercise the equal-code leaf collapse
    (lbvh-kernels.cu:316-331)."""
    z = load(golden_dir, "lbvh_cases.npz")
    for case in ("dup64", "clump"):
        nodes = z[f"{case}/nodes"]
        n = z[f"{case}/ids"].shape[0]
        inner = nodes[: n - 1, 0].view(np.uint32)
        assert ((inner & 1) == 0).sum() > 0


def _sphere_rays(z):
    o, d, m = O.shirley_rays(z["tan_half"], np.float32(np.float32(z["w"]) / np.float32(z["h"])),
                             int(z["w"]), int(z["h"]), z["cam_dir"], z["cam_pos"], z["cam_up"])
    return o, d, m


def test_camera_rays_match_reference(golden_dir):
    z = load(golden_dir, "sphere_trace.npz")
    o, d, m = _sphere_rays(z)
    rays = np.concatenate([o.reshape(-1, 3), d.reshape(-1, 3), m[:, None]], axis=1)
    assert sha(rays.astype(np.float32)) == str(z["rays_sha"])


@pytest.mark.parametrize("mode", list(MODES))
def test_trace_kernels_match_reference(golden_dir, mode):
    z = load(golden_dir, "sphere_trace.npz")
    tris = records(z["pos"])
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    o, d, m = _sphere_rays(z)
    hits, _, overflow = O.trace(lb.nodes, srt, o, d, m, MODES[mode], stack_limit=32)
    assert not overflow
    if mode == "cis":
        ref = z["cis_hits"]
        for f in ("t", "beta", "gamma"):
            np.testing.assert_array_equal(hits[f].view(np.uint32), ref[f].view(np.uint32))
        valid = ref["t"] != np.float32(S.FLT_MAX)
        np.testing.assert_array_equal(hits["ref"][valid], ref["ref"][valid])
    assert sha(hits) == str(z[f"{mode}_sha"])


def test_lbvh_trace_matches_cpu_plugin(golden_dir):
    """Closest hits of the LBVH (GPU-path algorithm) equal the reference CPU
    plugin's spatial-median BVH hits by original triangle id (config 1)."""
    z = load(golden_dir, "sphere_trace.npz")
    tris = records(z["pos"])
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    o, d, m = _sphere_rays(z)
    hits, _, _ = O.trace(lb.nodes, srt, o, d, m, O.CIS, stack_limit=32)
    valid = hits["t"] != np.float32(S.FLT_MAX)
    ids = np.where(valid, lb.ids[hits["ref"]], np.uint32(0xFFFFFFFF))
    np.testing.assert_array_equal(ids, z["bbvh_id"])
    np.testing.assert_array_equal(hits["t"].view(np.uint32), z["bbvh_t"].view(np.uint32))


def test_cpu_plugin_port_matches_reference(golden_dir):
    """The C port of bbvh.so (CPU baseline on machines without the reference
    sources) reproduces the reference plugin's hits."""
    z = load(golden_dir, "sphere_trace.npz")
    tris = records(z["pos"])
    nodes, leaf_tris = O.bbvh_build(tris)
    o, d, m = _sphere_rays(z)
    hits = O.bbvh_trace_cis(nodes, leaf_tris, o, d, m)
    valid = hits["t"] != np.float32(S.FLT_MAX)
    ids = np.where(valid, S.tag_ids(leaf_tris)[hits["ref"]], np.uint32(0xFFFFFFFF))
    np.testing.assert_array_equal(ids, z["bbvh_id"])
    np.testing.assert_array_equal(hits["t"].view(np.uint32), z["bbvh_t"].view(np.uint32))


@pytest.mark.parametrize("mode", ["cis", "dis"])
def test_terrain_trace_matches_reference(golden_dir, mode):
    z = load(golden_dir, "terrain_trace.npz")
    tris = records(z["pos"])
    lb = O.lbvh_build(tris, 30)
    np.testing.assert_array_equal(lb.codes.astype(np.uint32), z["codes"])
    np.testing.assert_array_equal(lb.ids, z["ids"])
    assert sha(lb.nodes) == str(z["nodes_sha"])
    srt = O.permute(tris, lb.ids)
    o, d, m = O.shirley_rays(z["tan_half"], np.float32(np.float32(z["w"]) / np.float32(z["h"])),
                             int(z["w"]), int(z["h"]), z["cam_dir"], z["cam_pos"], z["cam_up"])
    hits, _, _ = O.trace(lb.nodes, srt, o, d, m, MODES[mode], stack_limit=32)
    ref = z[f"{mode}_hits"]
    assert sha(hits) == sha(ref)


def test_shading_matches_reference_lighting_collector(golden_dir):
    """orc_shade_lambert against the reference's own lighting_collector
    (librta/raytrav.h:174-243) run on the sphere view's hits."""
    z = np.load(os.path.join(golden_dir, "shade_sphere.npz"))
    sp = np.load(os.path.join(golden_dir, "sphere_trace.npz"))
    hits = sp["cis_hits"].view(O.HIT_DTYPE)
    w, h = int(sp["w"]), int(sp["h"])
    img = O.shade_lambert(z["tris"], hits, w, h, z["lights"], False, z["bg"])
    np.testing.assert_array_equal(img, z["image"])
    img = O.shade_lambert(z["tris"], hits, w, h, z["lights"], True, z["bg"])
    np.testing.assert_array_equal(img, z["binary"])
    # the background of reset(c) on every miss, shading on every hit
    miss = hits["t"] == np.float32(np.finfo(np.float32).max)
    assert np.all(z["image"][miss.reshape(h, w)] == np.array([25, 51, 76], np.uint8))
    assert (~miss).sum() > 10000


def test_png_writer_round_trip(tmp_path):
    import struct
    import zlib
    from rta_gb300.plugin import write_png
    rgb = np.random.default_rng(0).integers(0, 256, size=(7, 5, 3), dtype=np.uint8)
    path = str(tmp_path / "x.png")
    write_png(path, rgb)
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (5, 7)
    idat_len = struct.unpack(">I", data[33:37])[0]
    raw = zlib.decompress(data[41:41 + idat_len])
    rows = np.frombuffer(raw, np.uint8).reshape(7, 1 + 5 * 3)
    assert np.all(rows[:, 0] == 0)
    np.testing.assert_array_equal(rows[:, 1:].reshape(7, 5, 3), rgb)
