"""GPU parity of the batched multi-mesh path: every mesh's tree (codes,
sorted ids, every 2F4 node word) equals the oracle's one-mesh LBVH, every
ray's hit equals the oracle's trace of its own mesh, the graph replay equals
the eager calls, every launch parameter gives the same results, and the
per-mesh sequential path gives the same hits."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402
from rta_gb300 import batch as B  # noqa: E402
from rta_gb300 import lib as L  # noqa: E402
from rta_gb300 import scenes as S  # noqa: E402


def hits_np(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(O.HIT_DTYPE)


def assert_hits_equal(a, b):
    """t of every ray; beta, gamma and ref of the rays that hit (a miss writes
    only t, so its other fields keep whatever the buffer held)."""
    np.testing.assert_array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32), err_msg="t")
    valid = a["t"] != np.float32(S.FLT_MAX)
    for f in ("beta", "gamma", "ref"):
        np.testing.assert_array_equal(a[f][valid].view(np.uint32), b[f][valid].view(np.uint32), err_msg=f)


def small_specs():
    """Twelve meshes of both kinds with 1k-9k triangles and 4k-30k rays."""
    specs = B.S.batch_specs(meshes=12, seed=3, total_tris=40_000, tri_range=(1000, 9000),
                            total_rays=120_000, ray_range=(4096, 30_000))
    return specs


def tiny_meshes(rng):
    """Meshes of 1, 2, 3 and 7 triangles and one of 64 identical triangles."""
    pos = [rng.uniform(-1, 1, size=(k, 3, 3)).astype(np.float32) for k in (1, 2, 3, 7)]
    dup = np.repeat(rng.uniform(-1, 1, size=(1, 3, 3)).astype(np.float32), 64, axis=0)
    out = [S._records(p[:, 0], p[:, 1], p[:, 2]) for p in pos + [dup]]
    return out


@pytest.fixture(scope="module")
def work():
    rng = np.random.default_rng(11)
    specs = small_specs()
    w = B.make_workload(specs)
    # prepend tiny meshes (with a few rays each, one of them with none)
    tiny = tiny_meshes(rng)
    tris = np.concatenate(tiny + [w.tris_host])
    tri_off = np.concatenate([[0], np.cumsum([t.shape[0] for t in tiny]), np.cumsum([t.shape[0] for t in tiny])[-1]
                              + w.tri_offsets[1:]]).astype(np.uint32)
    nr_tiny = [64, 0, 32, 64, 128]
    o, d, m = S.incoherent_rays(sum(nr_tiny), extent=2.0, seed=5)
    dev = torch.device("cuda")
    orig = torch.cat([torch.from_numpy(o).to(dev), w.orig])
    dirs = torch.cat([torch.from_numpy(d).to(dev), w.dirs])
    maxt = torch.cat([torch.from_numpy(m).to(dev), w.maxt])
    ray_off = np.concatenate([[0], np.cumsum(nr_tiny), sum(nr_tiny) + w.ray_offsets[1:]]).astype(np.uint32)
    w2 = B.Workload(None, np.ascontiguousarray(tris), tri_off, ray_off, orig, dirs, maxt)
    return w2


def meshes_of(w):
    return len(w.tri_offsets) - 1


def fresh_hits(n):
    return torch.from_numpy(O.reset_hits(n).view(np.float32).reshape(-1).copy()).to("cuda")


def test_every_mesh_tree_matches_the_oracle(work):
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    b.build(work.tris)
    assert b.status() & ~(L.DEV_QUANT_WRAP | L.DEV_ZERO_EXTENT) == 0
    for m in range(meshes_of(work)):
        lb = O.lbvh_build(work.mesh_tris(m), 30)
        mv = b.mesh(m)
        np.testing.assert_array_equal(mv.codes(), lb.codes.astype(np.uint32), err_msg=f"codes {m}")
        np.testing.assert_array_equal(mv.index_buffer, lb.ids, err_msg=f"ids {m}")
        np.testing.assert_array_equal(mv.node_data_2f4().view(np.uint32), lb.nodes.view(np.uint32),
                                      err_msg=f"nodes {m}")


def test_batch_trace_matches_the_oracle_per_mesh(work):
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    b.build(work.tris)
    hits = fresh_hits(work.n_rays)
    b.trace(work.orig, work.dirs, work.maxt, hits)
    got = hits_np(hits)
    for m in range(meshes_of(work)):
        a, e = int(work.ray_offsets[m]), int(work.ray_offsets[m + 1])
        if a == e:
            continue
        lb = O.lbvh_build(work.mesh_tris(m), 30)
        o, d, mx = (x.cpu().numpy() for x in work.mesh_rays(m))
        want, _, overflow = O.trace(lb.nodes, O.permute(work.mesh_tris(m), lb.ids), o, d, mx, O.CIS)
        assert not overflow
        assert_hits_equal(got[a:e], want)
    assert b.status() & ~(L.DEV_QUANT_WRAP | L.DEV_ZERO_EXTENT) == 0


def test_graph_run_matches_eager_and_replays(work):
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    b.build(work.tris)
    want = fresh_hits(work.n_rays)
    b.trace(work.orig, work.dirs, work.maxt, want)
    want = hits_np(want)
    hits = torch.zeros(4 * work.n_rays, dtype=torch.float32, device="cuda")
    for _ in range(3):   # capture, then two replays
        hits.zero_()
        b.run(work.tris, work.orig, work.dirs, work.maxt, hits)
        assert_hits_equal(hits_np(hits), want)


@pytest.mark.parametrize("params", [{"digit_bits": 10}, {"digit_bits": 11}, {"stack": 64},
                                    {"fetch_idle": 1}, {"fetch_idle": 32}, {"blocks_per_sm": 1}])
def test_every_launch_parameter_gives_the_same_results(work, params):
    ref = B.Batch()
    ref.set_meshes(work.tri_offsets, work.ray_offsets)
    h0 = torch.zeros(4 * work.n_rays, dtype=torch.float32, device="cuda")
    ref.run(work.tris, work.orig, work.dirs, work.maxt, h0)
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    b.params = params
    assert {k: b.params[k] for k in params} == params
    h1 = torch.zeros(4 * work.n_rays, dtype=torch.float32, device="cuda")
    b.run(work.tris, work.orig, work.dirs, work.maxt, h1)
    assert_hits_equal(hits_np(h1), hits_np(h0))
    for m in (0, 4, meshes_of(work) - 1):
        np.testing.assert_array_equal(b.mesh(m).node_data_2f4().view(np.uint32),
                                      ref.mesh(m).node_data_2f4().view(np.uint32))


def test_sequential_per_mesh_path_gives_the_same_hits(work):
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    h0 = torch.zeros(4 * work.n_rays, dtype=torch.float32, device="cuda")
    b.run(work.tris, work.orig, work.dirs, work.maxt, h0)
    h1 = torch.zeros(4 * work.n_rays, dtype=torch.float32, device="cuda")
    B.sequential(work, h1)
    # both reset as reset_intersections does, so even the misses' words agree
    np.testing.assert_array_equal(hits_np(h1).view(np.uint32), hits_np(h0).view(np.uint32))


def test_autotune_picks_valid_parameters_and_caches_them(work, tmp_path):
    cache = str(tmp_path / "tune.json")
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    hits = torch.zeros(4 * work.n_rays, dtype=torch.float32, device="cuda")
    chosen, ms = b.autotune(work.tris, work.orig, work.dirs, work.maxt, hits, cache_path=cache, reps=2)
    assert ms > 0
    assert chosen["digit_bits"] in (8, 9, 10, 11) and chosen["stack"] in (40, 64)
    assert b.params == chosen
    with open(cache) as f:
        entries = json.load(f)
    assert entries[b.tune_key()]["digit_bits"] == chosen["digit_bits"]
    # a second batch of the same workload takes the cached choice untimed
    b2 = B.Batch()
    b2.set_meshes(work.tri_offsets, work.ray_offsets)
    again, ms2 = b2.autotune(work.tris, work.orig, work.dirs, work.maxt, hits, cache_path=cache, reps=2)
    assert again == chosen and ms2 == -1.0
    # and the tuned parameters still give the reference hits
    want = fresh_hits(work.n_rays)
    B.sequential(work, want)
    b2.run(work.tris, work.orig, work.dirs, work.maxt, hits)
    assert_hits_equal(hits_np(hits), hits_np(want))
    assert os.path.getsize(cache) > 0


@pytest.mark.parametrize("digit_bits", [8, 9, 10, 11])
def test_one_mesh_builds_after_batch_builds(work, digit_bits):
    """A batch build and a one-mesh build of the same key width instantiate
    the same sort kernel in two translation units; each must launch its own
    (a shared launcher once left the one-mesh sort without its shared-memory
    attribute).  Both, run back to back, match the oracle."""
    from rta_gb300 import plugin as P
    b = B.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    b.params = {"digit_bits": digit_bits}
    b.build(work.tris)
    tris = S.clusters(16, 1024, seed=9)
    lb = O.lbvh_build(tris, 63)
    ctor = P.lbvh_constructor(morton_bits=63, digit_bits=digit_bits)
    bvh = ctor.build(P.cuda_ftl(tris))
    np.testing.assert_array_equal(bvh.node_data_2f4().view(np.uint32), lb.nodes.view(np.uint32))
    m = meshes_of(work) - 1
    lbm = O.lbvh_build(work.mesh_tris(m), 30)
    np.testing.assert_array_equal(b.mesh(m).node_data_2f4().view(np.uint32), lbm.nodes.view(np.uint32))
