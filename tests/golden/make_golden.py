"""Generates the golden fixtures in this folder from the reference itself.

Needs the reference sources ($RTA_REFERENCE, else a checkout beside this repository): the
recipe in oracle/refbuild compiles

* the reference CPU plugin bbvh.so (bbvh/) driven through rta's plugin ABI,
* the reference CUDA kernels (bbvh-cuda/lbvh-kernels.cu, bbvh-cuda/kernels.cu,
  librta/cuda-kernels.cu) run on the CPU by a launch emulation,

and this script feeds them seeded inputs and stores inputs and outputs:

* ``lbvh_cases.npz``   small LBVH builds (n = 1, 2, 3, 7, duplicates, random,
                       terrain, clusters, the 6,240-triangle sphere): Morton
                       codes, sorted ids, the 2F4 node array, the scene box.
* ``sphere_trace.npz`` the 256x256 sphere view (60 degree FOV): the reference
                       camera kernel's rays (digest) and the hits of the six
                       2F4 trace kernels, plus the CPU plugin's hits by
                       original triangle id.
* ``terrain_trace.npz`` a 64x32-quad terrain seen by a 160x90 camera: hits of
                       the CIS and DIS kernels.
* ``mamo_dumps.npz``   the reference's own mamo text dumps
                       (binary_bvh::dump_acceleration_structure / ::dump_primitives,
                       bbvh/bbvh.h:36-65; cam_ray_generator_shirley::dump_rays,
                       librta/raytrav.h:353-366) of a 256-triangle terrain's
                       reference LBVH, its triangles and a 16x4 ray image, with
                       nodes, triangles and rays of special values appended
                       (-0, +-inf, +-NaN, subnormal, integral and large values).

Run from the repository root:  python tests/golden/make_golden.py
(``python tests/golden/make_golden.py dumps`` remakes mamo_dumps.npz alone)
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from rta_gb300 import scenes as S  # noqa: E402

REF = os.environ.get("RTA_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
OUT = os.path.dirname(os.path.abspath(__file__))
REFDIR = os.path.join(ROOT, "oracle", "_ref")
HIT = np.dtype([("t", "<f4"), ("beta", "<f4"), ("gamma", "<f4"), ("ref", "<u4")])
MODES = ["cis", "dis", "shadow_cis", "shadow_dis", "cis_aila", "dis_aila"]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def records(pos: np.ndarray) -> np.ndarray:
    """(n, 9) positions -> reference records with material_index = triangle id."""
    p = pos.reshape(-1, 3, 3)
    return S._records(p[:, 0], p[:, 1], p[:, 2])


def positions(tris: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(tris[:, 0:9], np.float32)


def emu(tmp, *args):
    r = subprocess.run([os.path.join(REFDIR, "lbvh_emu"), *map(str, args)], capture_output=True,
                       text=True, cwd=tmp)
    if r.returncode != 0:
        raise RuntimeError(f"lbvh_emu {args[0]} failed: {r.stderr}")


def ref_lbvh(tmp, tris):
    n = tris.shape[0]
    tris.astype(np.float32).tofile(os.path.join(tmp, "t.f32"))
    emu(tmp, "lbvh", "t.f32", n, "e")
    rd = lambda ext, dt: np.fromfile(os.path.join(tmp, "e." + ext), dt)  # noqa: E731
    return dict(codes=rd("codes", np.uint32), ids=rd("ids", np.uint32),
                nodes=rd("nodes", np.float32).reshape(-1, 8), scene=rd("scene", np.float32),
                tris=rd("tris", np.float32).reshape(-1, 26))


def ref_trace(tmp, mode, lb, rays):
    n = lb["ids"].shape[0]
    lb["nodes"].tofile(os.path.join(tmp, "n.bin"))
    lb["tris"].tofile(os.path.join(tmp, "s.f32"))
    rays.astype(np.float32).tofile(os.path.join(tmp, "r.f32"))
    emu(tmp, "trace", mode, "n.bin", n, "s.f32", "r.f32", rays.shape[0], "h.bin")
    return np.fromfile(os.path.join(tmp, "h.bin"), HIT)


def ref_rays(tmp, cam: S.Camera):
    emu(tmp, "rays", cam.w, cam.h, cam.fovy, *cam.pos.tolist(), *cam.dir.tolist(),
        *cam.up.tolist(), "rays.bin")
    raw = np.fromfile(os.path.join(tmp, "rays.bin"), np.float32)
    return raw[:-1].reshape(-1, 7), np.float32(raw[-1])


def ref_bbvh(tmp, tris, rays, width):
    tris.astype(np.float32).tofile(os.path.join(tmp, "t.f32"))
    rays.astype(np.float32).tofile(os.path.join(tmp, "r.f32"))
    r = subprocess.run([os.path.join(REFDIR, "bbvh_harness"), os.path.join(REFDIR, "bbvh.so"),
                        "t.f32", str(tris.shape[0]), "r.f32", str(rays.shape[0]), "o.bin",
                        str(width)], capture_output=True, text=True, cwd=tmp)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    raw = np.fromfile(os.path.join(tmp, "o.bin"), np.uint8)
    return raw[:-4].view(np.dtype([("t", "<f4"), ("beta", "<f4"), ("gamma", "<f4"), ("id", "<u4")]))


def ref_shade(tmp, tris, hits, w, h, lights, binary, bg):
    """The reference's lighting_collector (librta/raytrav.h:174-243) run by
    oracle/refbuild/shade_harness.cpp."""
    tris.astype(np.float32).tofile(os.path.join(tmp, "st.f32"))
    np.ascontiguousarray(hits).tofile(os.path.join(tmp, "sh.bin"))
    lights.astype(np.float32).tofile(os.path.join(tmp, "sl.f32"))
    r = subprocess.run([os.path.join(REFDIR, "shade_harness"), "st.f32", str(tris.shape[0]), "sh.bin", str(w),
                        str(h), "sl.f32", str(lights.shape[0]), str(int(binary)), *map(str, bg), "img.rgb"],
                       capture_output=True, text=True, cwd=tmp)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return np.fromfile(os.path.join(tmp, "img.rgb"), np.uint8).reshape(h, w, 3)


LIGHTS = np.array([[2.0, 3.0, 4.0, 0.9, 0.8, 0.7], [-3.0, 1.0, 2.0, 0.2, 0.3, 0.5]], np.float32)
BACKGROUND = (0.1, 0.2, 0.3)


def small_cases():
    rng = np.random.default_rng(1234)
    cases = {}
    cases["n1"] = rng.uniform(-1, 1, (1, 9))
    cases["n2"] = rng.uniform(-1, 1, (2, 9))
    cases["n3"] = rng.uniform(-1, 1, (3, 9))
    cases["n7"] = rng.uniform(-1, 1, (7, 9))
    base = rng.uniform(-1, 1, (16, 9))
    dup = np.repeat(base, 4, axis=0)                      # equal centroids -> collapsed leaves
    cases["dup64"] = dup[rng.permutation(64)]
    cases["rand100"] = rng.uniform(-3, 5, (100, 9))
    clump = rng.normal(0, 1e-3, (40, 9)) + 0.5            # a dense clump: many equal codes
    cases["clump"] = np.concatenate([clump, rng.uniform(-1, 1, (24, 9))])
    cases["terrain16x8"] = positions(S.terrain(16, 8, seed=3))
    cases["clusters4x64"] = positions(S.clusters(4, 64, seed=5))
    cases["sphere"] = positions(S.uv_sphere())
    return {k: np.asarray(v, np.float32) for k, v in cases.items()}


SPECIALS = np.array([-0.0, np.inf, -np.inf, np.nan, -np.nan, 1e-7, 123456789.0, 0.1, 3.0, 1e20, 5e-39,
                     -2.5, 65536.0, 1.0 / 3.0], np.float32)
SPECIALS[4] = np.float32(np.copysign(np.float32(np.nan), -1.0))   # NaN with the sign bit set


def dump_inputs():
    """The arrays whose dumps are pinned: a 16x8-quad terrain's reference
    LBVH (2F4 nodes) and Morton-ordered triangles, a 16x4 ray image of the
    terrain camera, and records of special values appended to each."""
    from oracle import oracle as O
    tris = S.terrain(16, 8, seed=3)
    lb = O.lbvh_build(tris, 30)
    nodes = np.asarray(lb.nodes, np.float32).reshape(-1, 8).copy()
    srt = np.asarray(O.permute(tris, lb.ids), np.float32).reshape(-1, 26).copy()
    sp = SPECIALS
    extra_nodes = np.zeros((4, 8), np.float32)
    words = np.array([[(7 << 1) | 1, 9], [3 << 1, 250], [0, 0], [(1 << 24) << 1 | 1, 4000000000]], np.uint32)
    extra_nodes[:, :2] = words.view(np.float32)
    extra_nodes[:, 2:] = np.resize(sp, (4, 6))
    extra_tris = np.resize(sp, (3, 26)).astype(np.float32)
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=16, h=4)
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    rays = np.concatenate([np.asarray(o, np.float32).reshape(-1, 3), np.asarray(d, np.float32).reshape(-1, 3),
                           np.asarray(m, np.float32).reshape(-1, 1)], axis=1)
    rays[-3:, :] = np.resize(sp, (3, 7))
    return np.concatenate([nodes, extra_nodes]), np.concatenate([srt, extra_tris]), rays, cam.w, cam.h


def ref_dumps(tmp, nodes, tris, rays, w, h):
    np.ascontiguousarray(nodes, np.float32).tofile(os.path.join(tmp, "dn.f32"))
    np.ascontiguousarray(tris, np.float32).tofile(os.path.join(tmp, "dt.f32"))
    np.ascontiguousarray(rays, np.float32).tofile(os.path.join(tmp, "dr.f32"))
    prefix = os.path.join(tmp, "dump")
    subprocess.run([os.path.join(REFDIR, "dump_harness"), os.path.join(tmp, "dn.f32"), str(nodes.shape[0]),
                    os.path.join(tmp, "dt.f32"), str(tris.shape[0]), os.path.join(tmp, "dr.f32"), str(w), str(h),
                    prefix], check=True)
    out = {}
    for ext in ("bvh", "tri", "ray"):
        with open(f"{prefix}.{ext}", "rb") as f:
            out[ext] = np.frombuffer(f.read(), np.uint8)
    return out


def make_dumps(tmp):
    nodes, tris, rays, w, h = dump_inputs()
    txt = ref_dumps(tmp, nodes, tris, rays, w, h)
    np.savez_compressed(os.path.join(OUT, "mamo_dumps.npz"), nodes=nodes, tris=tris, rays=rays, w=w, h=h,
                        bvh_text=txt["bvh"], tri_text=txt["tri"], ray_text=txt["ray"])


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "refbuild"), f"REF={REF}"],
                   check=True)
    if len(sys.argv) > 1 and sys.argv[1] == "dumps":
        with tempfile.TemporaryDirectory() as tmp:
            make_dumps(tmp)
        print("mamo_dumps.npz", os.path.getsize(os.path.join(OUT, "mamo_dumps.npz")))
        return
    with tempfile.TemporaryDirectory() as tmp:
        out = {}
        for name, pos in small_cases().items():
            lb = ref_lbvh(tmp, records(pos))
            out[f"{name}/pos"] = pos
            out[f"{name}/codes"] = lb["codes"]
            out[f"{name}/ids"] = lb["ids"]
            out[f"{name}/nodes"] = lb["nodes"]
            out[f"{name}/scene"] = lb["scene"]
        np.savez_compressed(os.path.join(OUT, "lbvh_cases.npz"), **out)

        # config-1 view of the sphere
        sphere = records(positions(S.uv_sphere()))
        lb = ref_lbvh(tmp, sphere)
        cam = S.sphere_camera()
        rays, tanv = ref_rays(tmp, cam)
        sp = dict(pos=positions(sphere), tan_half=np.float32(tanv), w=cam.w, h=cam.h,
                  cam_pos=cam.pos, cam_dir=cam.dir, cam_up=cam.up,
                  rays_sha=sha(rays))
        for mode in MODES:
            hits = ref_trace(tmp, mode, lb, rays)
            sp[f"{mode}_sha"] = sha(hits)
            if mode == "cis":
                sp["cis_hits"] = hits
        cpu = ref_bbvh(tmp, sphere, rays, cam.w)
        sp["bbvh_t"] = cpu["t"]
        sp["bbvh_id"] = cpu["id"]
        np.savez_compressed(os.path.join(OUT, "sphere_trace.npz"), **sp)

        # host shading of that view, with the sphere's own vertex normals (same
        # positions, so the same tree and hits)
        smooth = S.uv_sphere()
        lbs = ref_lbvh(tmp, smooth)
        assert np.array_equal(lbs["ids"], lb["ids"])
        sh = dict(lights=LIGHTS, bg=np.asarray(BACKGROUND, np.float32), tris=lbs["tris"],
                  image=ref_shade(tmp, lbs["tris"], sp["cis_hits"], cam.w, cam.h, LIGHTS, False, BACKGROUND),
                  binary=ref_shade(tmp, lbs["tris"], sp["cis_hits"], cam.w, cam.h, LIGHTS, True, BACKGROUND))
        np.savez_compressed(os.path.join(OUT, "shade_sphere.npz"), **sh)

        # a small terrain view
        ter = records(positions(S.terrain(64, 32, seed=11)))
        lb = ref_lbvh(tmp, ter)
        tcam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=160, h=90)
        rays, tanv = ref_rays(tmp, tcam)
        tt = dict(pos=positions(ter), tan_half=np.float32(tanv), w=tcam.w, h=tcam.h,
                  cam_pos=tcam.pos, cam_dir=tcam.dir, cam_up=tcam.up, rays_sha=sha(rays),
                  codes=lb["codes"], ids=lb["ids"], nodes_sha=sha(lb["nodes"]))
        for mode in ("cis", "dis"):
            tt[f"{mode}_hits"] = ref_trace(tmp, mode, lb, rays)
        np.savez_compressed(os.path.join(OUT, "terrain_trace.npz"), **tt)
        make_dumps(tmp)
    for f in ("lbvh_cases.npz", "sphere_trace.npz", "terrain_trace.npz", "shade_sphere.npz", "mamo_dumps.npz"):
        print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
