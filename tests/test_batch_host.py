"""Host-side logic of the batched path, without a device: the tuning cache
(written and read by the library, parsed as JSON here), argument checks that
happen before any device call, and the batched workload generator."""
import ctypes as C
import json

import numpy as np
import pytest

from rta_gb300 import batch as B
from rta_gb300 import lib as L
from rta_gb300 import scenes as S


@pytest.fixture(scope="module")
def lib():
    return L.load()


def test_tune_cache_round_trip(tmp_path):
    path = str(tmp_path / "cache.json")
    assert B.tune_cache_lookup(path, "gpu|sm152|meshes512") is None   # no file yet
    p1 = {"digit_bits": 8, "fetch_idle": 12, "blocks_per_sm": 0, "stack": 40}
    p2 = {"digit_bits": 10, "fetch_idle": 4, "blocks_per_sm": 6, "stack": 64}
    B.tune_cache_store(path, "gpu|sm152|meshes512", p1, 3.5)
    B.tune_cache_store(path, "gpu|sm152|meshes16", p2, 0.25)
    assert B.tune_cache_lookup(path, "gpu|sm152|meshes512") == p1
    assert B.tune_cache_lookup(path, "gpu|sm152|meshes16") == p2
    assert B.tune_cache_lookup(path, "gpu|sm152|meshes1") is None
    # replacing an entry keeps the others, and the file stays valid JSON
    p3 = dict(p1, fetch_idle=24)
    B.tune_cache_store(path, "gpu|sm152|meshes512", p3, 3.25)
    with open(path) as f:
        d = json.load(f)
    assert set(d) == {"gpu|sm152|meshes512", "gpu|sm152|meshes16"}
    assert d["gpu|sm152|meshes512"]["fetch_idle"] == 24 and d["gpu|sm152|meshes512"]["ms"] == 3.25
    assert B.tune_cache_lookup(path, "gpu|sm152|meshes512") == p3


def test_tune_cache_rejects_bad_keys_and_parameters(tmp_path, lib):
    path = str(tmp_path / "cache.json").encode()
    ok = L.BatchParams(8, 12, 0, 40)
    assert lib.rta_tune_cache_store(path, b'bad"key', C.byref(ok), 1.0) == L.ERR_INVALID
    assert lib.rta_tune_cache_store(path, b"", C.byref(ok), 1.0) == L.ERR_INVALID
    for bad in (L.BatchParams(12, 12, 0, 40), L.BatchParams(8, 0, 0, 40), L.BatchParams(8, 33, 0, 40),
                L.BatchParams(8, 12, -1, 40), L.BatchParams(8, 12, 0, 48)):
        assert lib.rta_tune_cache_store(path, b"k", C.byref(bad), 1.0) == L.ERR_INVALID


def test_batch_arguments_are_checked_before_the_device(lib):
    h = C.c_void_p()
    assert lib.rta_batch_create(C.byref(h)) == L.OK
    try:
        def off(a):
            return np.ascontiguousarray(a, np.uint32).ctypes.data_as(C.c_void_p)
        t_ok, r_ok = np.array([0, 3, 7], np.uint32), np.array([0, 0, 5], np.uint32)
        assert lib.rta_batch_set_meshes(h, 0, off(t_ok), off(r_ok)) == L.ERR_INVALID
        assert lib.rta_batch_set_meshes(h, 2, off([1, 3, 7]), off(r_ok)) == L.ERR_INVALID   # must start at 0
        assert lib.rta_batch_set_meshes(h, 2, off([0, 3, 3]), off(r_ok)) == L.ERR_INVALID   # empty mesh
        assert lib.rta_batch_set_meshes(h, 2, off(t_ok), off([0, 5, 2])) == L.ERR_INVALID   # rays go back
        big = lib.rta_lbvh_max_triangles() + 1
        assert lib.rta_batch_set_meshes(h, 2, off([0, 3, 3 + big]), off(r_ok)) == L.ERR_INVALID
        assert lib.rta_batch_build(h, C.c_void_p(16), None) == L.ERR_INVALID   # no meshes yet
        assert lib.rta_batch_trace(h, None, None, None, None, None, None) == L.ERR_INVALID   # not built
        v = L.LbvhView()
        assert lib.rta_batch_mesh(h, 0, C.byref(v)) == L.ERR_INVALID
        for bad in (L.BatchParams(7, 12, 0, 40), L.BatchParams(8, 12, 0, 32), L.BatchParams(8, 40, 0, 40)):
            assert lib.rta_batch_set_params(h, C.byref(bad)) == L.ERR_INVALID
        good = L.BatchParams(11, 4, 2, 64)
        assert lib.rta_batch_set_params(h, C.byref(good)) == L.OK
        back = L.BatchParams()
        assert lib.rta_batch_get_params(h, C.byref(back)) == L.OK
        assert back.as_dict() == good.as_dict()
    finally:
        assert lib.rta_batch_destroy(h) == L.OK


def test_batch_workload_sizes():
    specs = S.batch_specs()   # the 512-mesh workload
    nt = np.array([s.n_tris for s in specs])
    nr = np.array([s.n_rays for s in specs])
    assert len(specs) == 512
    assert nt.min() >= 1000 and nt.max() <= 200_000
    assert abs(int(nt.sum()) - 25_000_000) < 25_000
    assert nr.min() >= 4096 and nr.max() <= 1 << 20
    assert {s.kind for s in specs} == {"terrain", "clusters"}
    for s in specs:
        assert 0 < s.n_primary <= s.n_rays // 2 + 1
        assert s.cam.w * s.cam.h == s.n_primary
    # the same seed gives the same workload; meshes have exactly their count
    again = S.batch_specs()
    assert [(s.kind, s.n_tris, s.n_rays) for s in again] == [(s.kind, s.n_tris, s.n_rays) for s in specs]
    small = [s for s in specs if s.n_tris < 3000][:2] + [s for s in specs if s.kind == "terrain"][:1]
    for s in small:
        assert S.batch_mesh_triangles(s).shape == (s.n_tris, S.TRI_FLOATS)
