"""The learned child order: the recording traversal is the plain one, samples
are labelled by the final hit, the tensor-core gradient equals the CPU
restatement, training lowers the loss, and the learned order keeps every
closest hit (t bit for bit; a different triangle only at an exact tie)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402
from rta_gb300 import learned as LR  # noqa: E402
from rta_gb300 import plugin as P  # noqa: E402
from rta_gb300 import scenes as S  # noqa: E402


@pytest.fixture(scope="module")
def terrain_case():
    tris = S.terrain(256, 128, seed=3)
    ctor = P.lbvh_constructor(morton_bits=30)
    bvh = ctor.build(P.cuda_ftl(tris))
    bvh._ctor = ctor
    cam = S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=640, h=360)
    g = P.cam_ray_generator_shirley(cam.w, cam.h)
    g.setup(cam.pos, cam.dir, cam.up, cam.fovy)
    g.generate_rays()
    return tris, bvh, g


@pytest.fixture(scope="module")
def cluster_case():
    tris = S.clusters(32, 2048, seed=4)
    ctor = P.lbvh_constructor(morton_bits=63)
    bvh = ctor.build(P.cuda_ftl(tris))
    bvh._ctor = ctor
    o, d, m = S.incoherent_rays(200_000, seed=4)
    dev = torch.device("cuda")
    return tris, bvh, (torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev), torch.from_numpy(m).to(dev))


def hits_np(h):
    return h.cpu().numpy().view(O.HIT_DTYPE)


def test_recording_trace_is_the_plain_trace(terrain_case):
    _, bvh, g = terrain_case
    model = LR.OrderModel(max_samples=1 << 20, seed=1)
    rec = model.sample(bvh, g.gpu_origin, g.gpu_direction, g.gpu_maxt)
    plain = LR.plain_trace(bvh, g.gpu_origin, g.gpu_direction, g.gpu_maxt)
    torch.cuda.synchronize()
    assert np.array_equal(rec.cpu().numpy().view(np.uint32), plain.cpu().numpy().view(np.uint32))
    assert model.sample_count() > 0


def test_samples_are_labelled_by_the_final_hit(terrain_case):
    _, bvh, g = terrain_case
    model = LR.OrderModel(max_samples=1 << 20, seed=1)
    hits = hits_np(model.sample(bvh, g.gpu_origin, g.gpu_direction, g.gpu_maxt))
    smp = model.samples().view(O.SAMPLE_DTYPE)
    assert smp.shape[0] == model.sample_count()
    ref = hits["ref"][smp["ray"]]
    hit = hits["t"][smp["ray"]] != np.float32(S.FLT_MAX)
    in_l = hit & (ref - smp["lfirst"] < smp["lsize"])
    in_r = hit & ~in_l & (ref - smp["rfirst"] < smp["rsize"])
    # weight: bit length of the other child's triangle count
    bitlen = lambda v: np.frexp(v.astype(np.float64))[1].astype(np.float32)
    want_w = np.where(in_l, bitlen(smp["rsize"]), np.where(in_r, bitlen(smp["lsize"]), 0.0))
    np.testing.assert_array_equal(smp["weight"], want_w.astype(np.float32))
    np.testing.assert_array_equal(smp["label"], in_l.astype(np.float32))
    # the two children's ranges are disjoint and adjacent (Karras split)
    lo = np.minimum(smp["lfirst"], smp["rfirst"])
    assert np.all(smp["lfirst"] + smp["lsize"] == smp["rfirst"])
    assert lo.size > 0


def test_gradient_matches_cpu_restatement(terrain_case):
    _, bvh, g = terrain_case
    model = LR.OrderModel(max_samples=1 << 20, seed=7)
    model.sample(bvh, g.gpu_origin, g.gpu_direction, g.gpu_maxt)
    n = min(8192, model.sample_count())
    grad, loss = model.gradient(0, n)
    smp = model.samples(n).view(O.SAMPLE_DTYPE)
    x = O.bf16_bits_to_f32(smp["x"].reshape(n, 16))
    ref, ref_loss = O.mlp_gradient(model.params(), x, smp["label"], smp["weight"], 1.0 / n)
    scale = np.abs(ref).max()
    assert np.abs(grad - ref).max() <= 2e-3 * scale, np.abs(grad - ref).max() / scale
    assert abs(loss - ref_loss / n) <= 1e-3 * abs(ref_loss / n)


def test_training_lowers_the_loss(terrain_case):
    _, bvh, g = terrain_case
    model = LR.OrderModel(max_samples=1 << 21, seed=3)
    model.sample(bvh, g.gpu_origin, g.gpu_direction, g.gpu_maxt)
    n = model.sample_count()
    _, before = model.gradient(0, n)
    after = model.train(epochs=4, batch=1 << 14, lr=3e-3)
    _, now = model.gradient(0, n)
    assert now < before
    assert np.isfinite(after)


@pytest.mark.parametrize("case", ["terrain", "clusters"])
def test_learned_order_keeps_closest_hits(case, terrain_case, cluster_case):
    if case == "terrain":
        _, bvh, g = terrain_case
        o, d, m = g.gpu_origin, g.gpu_direction, g.gpu_maxt
    else:
        _, bvh, (o, d, m) = cluster_case
    model = LR.OrderModel(max_samples=1 << 21, seed=5)
    model.sample(bvh, o, d, m)
    model.train(epochs=3, batch=1 << 14, lr=3e-3)
    got, st = model.trace(bvh, o, d, m, stats=True)
    want, sp = LR.plain_trace(bvh, o, d, m, stats=True)
    torch.cuda.synchronize()
    a, b = hits_np(got), hits_np(want)
    hit = b["t"] != np.float32(S.FLT_MAX)
    # a ray hits under either order, and t agrees to 1e-5 relative: a child is
    # culled once its rounded entry distance reaches the current t, and a
    # triangle's rounded t can lie a few ulps below its box's entry, so which
    # of two hits a few ulps apart survives can depend on the order
    np.testing.assert_array_equal(hit, a["t"] != np.float32(S.FLT_MAX))
    rel = np.abs(a["t"][hit].astype(np.float64) - b["t"][hit]) / np.abs(b["t"][hit])
    assert rel.max(initial=0.0) <= 1e-5
    assert (a["t"] != b["t"]).mean() < 1e-3
    ties = hit & (a["ref"] != b["ref"])
    assert ties.mean() < 1e-3   # ties and those ulp cases may report another triangle
    assert bvh.status() & 0x3F & ~0xC == 0


def _plain_rule_params(model):
    """Weights whose logit is feature 13, the plain rule's choice (+1 left
    first, -1 right first): h1 = relu(+-x13), h2 = h1, logit = h2[0] - h2[1]."""
    p = np.zeros_like(model.params())
    hid, inp = 32, 16
    w1 = p[: hid * inp].reshape(hid, inp)
    w1[0, 13], w1[1, 13] = 1.0, -1.0
    off_w2 = hid * inp + hid
    w2 = p[off_w2: off_w2 + hid * hid].reshape(hid, hid)
    w2[0, 0] = w2[1, 1] = 1.0
    off_w3 = off_w2 + hid * hid + hid
    p[off_w3 + 0], p[off_w3 + 1] = 1.0, -1.0
    return p


@pytest.mark.parametrize("case", ["terrain", "clusters"])
def test_inference_reproduces_a_known_rule(case, terrain_case, cluster_case):
    """With weights that output the plain rule's own choice, the fused
    tensor-core inference must pick exactly the plain order at every
    decision: every hit and every ray's node and triangle counts equal those
    of the plain traversal.  A huge margin (the network never overrides)
    gives the plain traversal for any weights."""
    if case == "terrain":
        _, bvh, g = terrain_case
        o, d, m = g.gpu_origin, g.gpu_direction, g.gpu_maxt
    else:
        _, bvh, (o, d, m) = cluster_case
    want, sp = LR.plain_trace(bvh, o, d, m, stats=True)
    model = LR.OrderModel(max_samples=1 << 10, seed=2)
    model.set_params(_plain_rule_params(model))
    assert model.margin() == 0.0
    got, st = model.trace(bvh, o, d, m, stats=True)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy().view(np.uint32), want.cpu().numpy().view(np.uint32))
    np.testing.assert_array_equal(st.cpu().numpy(), sp.cpu().numpy())
    # the opposite rule (logit = -x13) visits more nodes with the same hits
    anti_p = _plain_rule_params(model)
    off_w3 = 32 * 16 + 32 + 32 * 32 + 32
    anti_p[off_w3], anti_p[off_w3 + 1] = -1.0, 1.0
    model.set_params(anti_p)
    anti, sa = model.trace(bvh, o, d, m, stats=True)
    assert int(sa.sum()) > int(sp.sum())
    hit = hits_np(want)["t"] != np.float32(S.FLT_MAX)
    np.testing.assert_array_equal(hits_np(anti)["t"] != np.float32(S.FLT_MAX), hit)
    # random weights under a margin no logit reaches: the plain traversal
    # again, through the network kernel (3e38) and through the plain kernel
    # that FLT_MAX selects
    model2 = LR.OrderModel(max_samples=1 << 10, seed=9)
    for margin in (3.0e38, float(np.finfo(np.float32).max)):
        model2.set_margin(margin)
        got2, st2 = model2.trace(bvh, o, d, m, stats=True)
        assert np.array_equal(got2.cpu().numpy().view(np.uint32), want.cpu().numpy().view(np.uint32))
        np.testing.assert_array_equal(st2.cpu().numpy(), sp.cpu().numpy())
