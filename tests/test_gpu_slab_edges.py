"""The traversal's division-free slab decisions (trace.cu slab_bounds /
cis_decide / entry_axis) against the reference's exact slab test
(librta/intersect.h:56-150, restated by the oracle) on inputs aimed at the
edges of the filter's error bound, where a wrong bound would change which
child is visited first or whether a box counts as hit:

* lattice scenes whose LBVH boxes share planes (sibling boxes with the same
  entry plane, entries equal or a few ulps apart);
* rays whose origin lies exactly on slab planes, rays through lattice edges
  and corners (ties between sibling entries);
* direction components at, just inside and just outside the filter's
  |d| in [2^-100, 2^100] range, +-0 and one or two zero components;
* a lattice 1e2 units wide placed 1e6 from the origin, seen from nearby, so
  the |o * (1/d)| error term dominates the quotient's own;
* a lattice 1e-17 wide near the origin with huge direction components, so
  box quotients are subnormal or underflow to zero (no triangle of it can
  be hit: the triangle test's numerators underflow, in the reference too).

Every hit (t, beta, gamma, ref) and every ray's count of inner nodes visited
and triangles tested must equal the oracle's, for the child-is and the
direct-is order.  The corpus is generated here, seeded."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import oracle as O  # noqa: E402
from rta_gb300 import lib as L  # noqa: E402
from rta_gb300 import plugin as P  # noqa: E402
from rta_gb300 import scenes as S  # noqa: E402

F32 = np.float32
D_LO = F32(2.0 ** -100)   # the filter's range of |d|
D_HI = F32(2.0 ** 100)


def lattice(nx, ny, nz, scale=1.0, offset=(0.0, 0.0, 0.0)):
    """Unit squares (two triangles each) on the planes of an integer grid in
    all three orientations, scaled and shifted: many LBVH boxes share planes."""
    quads = []
    for k in range(nz + 1):          # z-planes
        for i in range(nx):
            for j in range(ny):
                if (i + j + k) % 2 == 0:
                    quads.append([(i, j, k), (i + 1, j, k), (i + 1, j + 1, k), (i, j + 1, k)])
    for i in range(0, nx + 1, 2):    # x-planes
        for j in range(ny):
            for k in range(nz):
                quads.append([(i, j, k), (i, j + 1, k), (i, j + 1, k + 1), (i, j, k + 1)])
    for j in range(0, ny + 1, 3):    # y-planes
        for i in range(nx):
            for k in range(nz):
                if (i + k) % 2 == 1:
                    quads.append([(i, j, k), (i + 1, j, k), (i + 1, j, k + 1), (i, j, k + 1)])
    q = np.asarray(quads, np.float64) * scale + np.asarray(offset, np.float64)
    q = q.astype(F32)
    a = np.concatenate([q[:, 0], q[:, 0]])
    b = np.concatenate([q[:, 1], q[:, 2]])
    c = np.concatenate([q[:, 2], q[:, 3]])
    return S._records(a, b, c)


def edge_directions(rng, n):
    """Directions with components at the filter's range limits and their
    float neighbours, +-0, and one or two zero components."""
    specials = np.array([0.0, -0.0, D_LO, np.nextafter(D_LO, F32(0)), np.nextafter(D_LO, F32(1)),
                         -D_LO, D_HI, np.nextafter(D_HI, F32(0)), np.nextafter(D_HI, F32(np.inf)), -D_HI,
                         F32(1e-20), F32(-3e-25), F32(1e25), F32(-7e28)], F32)
    d = rng.normal(size=(n, 3)).astype(F32)
    pick = rng.integers(0, 3, size=n)
    d[np.arange(n), pick] = specials[rng.integers(0, specials.size, size=n)]
    two = rng.random(n) < 0.2
    other = (pick + 1 + rng.integers(0, 2, size=n)) % 3
    d[two, other[two]] = specials[rng.integers(0, 2, size=int(two.sum()))]   # a second +-0
    return d


def corpus(scene, seed):
    """(tris, orig, dir, maxt) of one adversarial case."""
    rng = np.random.default_rng(seed)
    if scene == "lattice":
        tris = lattice(12, 12, 4)
        n = 1 << 16
        o = rng.uniform(-2.0, 14.0, size=(n, 3)).astype(F32)
        # a third of the origins lie exactly on slab planes
        on = rng.random((n, 3)) < 0.35
        o[on] = np.round(o[on])
        # a third aims exactly at lattice points: ties between sibling entries
        tgt = rng.integers(0, 13, size=(n, 3)).astype(F32)
        tgt[:, 2] = rng.integers(0, 5, size=n)
        d = (tgt - o).astype(F32)
        d[n // 3:2 * n // 3] = edge_directions(rng, 2 * n // 3 - n // 3)
        d[2 * n // 3:] = rng.normal(size=(n - 2 * n // 3, 3)).astype(F32)
    elif scene == "far":
        off = (1.0e6, -1.0e6, 3.0e5)
        tris = lattice(10, 10, 3, scale=10.0, offset=off)
        n = 1 << 15
        o = (np.asarray(off, np.float64) + rng.uniform(-20.0, 120.0, size=(n, 3))).astype(F32)
        tgt = (np.asarray(off, np.float64) + 10.0 * rng.integers(0, 11, size=(n, 3))).astype(F32)
        d = (tgt - o).astype(F32)
        d[n // 2:] = edge_directions(rng, n - n // 2)
    else:   # "tiny": quotients near or below the smallest normal float
        tris = lattice(8, 8, 2, scale=1e-18)
        n = 1 << 15
        o = (rng.uniform(-1.0, 9.0, size=(n, 3)) * 1e-18).astype(F32)
        on = rng.random((n, 3)) < 0.3
        o[on] = (np.round(o[on] / F32(1e-18)) * F32(1e-18)).astype(F32)
        d = rng.normal(size=(n, 3)).astype(F32) * F32(1e29)
        d[n // 2:] = edge_directions(rng, n - n // 2)
    m = np.full(o.shape[0], np.finfo(F32).max, F32)
    m[::7] = F32(5.0) if scene == "lattice" else m[::7]   # some finite max_t
    return tris, o.reshape(-1), d.reshape(-1), m


def gpu(tris, bits, o, d, m, mode):
    ctor = P.lbvh_constructor(morton_bits=bits)
    bvh = ctor.build(P.cuda_ftl(tris))
    dev = torch.device("cuda")
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a, F32)).to(dev)  # noqa: E731
    n = m.shape[0]
    h = torch.from_numpy(O.reset_hits(n).view(F32).reshape(-1).copy()).to(dev)
    st = torch.zeros(2 * n, dtype=torch.int32, device=dev)
    to_o, to_d, to_m = to(o), to(d), to(m)
    import ctypes as C
    L.check(L.load().rta_trace(C.byref(bvh.view), P._ptr(to_o), P._ptr(to_d), P._ptr(to_m), n, None, P._ptr(h),
                               mode | L.TRACE_STATS, P._ptr(st), P._stream()), "rta_trace")
    torch.cuda.synchronize()
    flags = bvh.status()
    return h.cpu().numpy().view(O.HIT_DTYPE), st.cpu().numpy().view(np.uint32).reshape(-1, 2), flags


@pytest.mark.parametrize("scene", ["lattice", "far", "tiny"])
@pytest.mark.parametrize("mode", ["cis", "dis"])
@pytest.mark.parametrize("bits", [30, 63])
def test_slab_decisions_at_the_error_bound_edges(scene, mode, bits):
    tris, o, d, m = corpus(scene, seed={"lattice": 1, "far": 2, "tiny": 3}[scene] + bits)
    lb = O.lbvh_build(tris, bits)
    om = O.CIS if mode == "cis" else O.DIS
    want, st_want, overflow = O.trace(lb.nodes, O.permute(tris, lb.ids), o, d, m, om, 128, stats=True)
    assert not overflow
    got, st_got, flags = gpu(tris, bits, o, d, m, L.TRACE_CIS if mode == "cis" else L.TRACE_DIS)
    assert flags & (L.DEV_STACK_OVERFLOW | L.DEV_ITER_LIMIT | L.DEV_BAD_LINK) == 0
    for f in ("t", "beta", "gamma"):
        np.testing.assert_array_equal(got[f].view(np.uint32), want[f].view(np.uint32), err_msg=f)
    valid = want["t"] != np.finfo(F32).max
    np.testing.assert_array_equal(got["ref"][valid], want["ref"][valid])
    np.testing.assert_array_equal(st_got, st_want)   # the same nodes and triangles, in the same order's count
    if scene == "tiny":
        # triangles this small never pass the triangle test (its numerators
        # underflow), but every ray walks many boxes on subnormal quotients
        assert st_want[:, 0].mean() > 20
    else:
        assert valid.mean() > 0.02


def filter_uncertain_fraction(tris, o, d, bits):
    """Share of (ray, root box) tests in which the filter's interval for t_near
    or t_far straddles a decision threshold of 0 or the other bound (the
    filter's arithmetic emulated in float64 and rounded to float32): the
    corpus drives the uncertain branch, where natural rays almost never go."""
    lb = O.lbvh_build(tris, bits)
    nodes = np.asarray(lb.nodes, F32).reshape(-1, 8)
    np.seterr(all="ignore")
    o = o.reshape(-1, 3).astype(np.float64)
    d = d.reshape(-1, 3).astype(F32)
    ok = np.all((np.abs(d) >= D_LO) & (np.abs(d) <= D_HI), axis=1)
    rd = (1.0 / d.astype(np.float64)).astype(F32).astype(np.float64)
    ord_ = (o * rd).astype(F32).astype(np.float64)
    eabs = np.max(np.abs(ord_), axis=1) * 2.0 ** -23 + 2.0 ** -146
    cnt = 0
    tot = 0
    for node in nodes[: min(64, nodes.shape[0])]:
        lo, hi = node[2:5].astype(np.float64), node[5:8].astype(np.float64)
        q1 = (lo * rd - ord_).astype(F32).astype(np.float64)
        q2 = (hi * rd - ord_).astype(F32).astype(np.float64)
        tn = np.max(np.minimum(q1, q2), axis=1)
        tf = np.min(np.maximum(q1, q2), axis=1)
        wn = np.abs(tn) * 2.0 ** -21 + eabs
        wf = np.abs(tf) * 2.0 ** -21 + eabs
        unc = ((tn - wn <= tf + wf) & (tn + wn > tf - wf)) | ((tf - wf < 0) & (tf + wf >= 0))
        cnt += int((unc & ok).sum())
        tot += int(ok.sum())
    return cnt / max(tot, 1)


def test_corpus_reaches_the_uncertain_branch():
    """Not a GPU check: the lattice corpus puts several per cent of its box
    tests into the filter's uncertain band (natural rays: about 0.03 %)."""
    tris, o, d, _ = corpus("lattice", seed=31)
    assert filter_uncertain_fraction(tris, o, d, 30) > 0.01
