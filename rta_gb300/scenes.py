"""Seeded synthetic scenes and ray sets for the LBVH build + trace workloads.

Triangles come back as ``(n, 26)`` float32 arrays: one row per reference
``cuda::simple_triangle`` record (librta/cuda-vec.h:30-37, 104 bytes): vertex
positions a, b, c, vertex normals na, nb, nc, texture coordinates ta, tb, tc
and the int ``material_index`` (raw bits in column 24; column 25 is the
struct's alignment padding).

The heightfield noise and the jitter use only integer hashing and IEEE
+,-,*,/ in float64 before the final cast, so a scene is the same on x86 and
Arm hosts.  The sphere and cluster generators use numpy's sin/cos; tests that
need bit-identical inputs across machines store their triangles.
"""
from __future__ import annotations

import math

import numpy as np

TRI_FLOATS = 26
FLT_MAX = float(np.finfo(np.float32).max)


def _records(a, b, c, na=None, nb=None, nc=None, uv=None, material=None) -> np.ndarray:
    n = a.shape[0]
    out = np.zeros((n, TRI_FLOATS), np.float32)
    out[:, 0:3] = a
    out[:, 3:6] = b
    out[:, 6:9] = c
    if na is not None:
        out[:, 9:12] = na
        out[:, 12:15] = nb
        out[:, 15:18] = nc
    if uv is not None:
        out[:, 18:24] = uv
    mat = np.arange(n, dtype=np.uint32) if material is None else np.asarray(material, np.uint32)
    out[:, 24] = mat.view(np.float32)
    return out


def tag_ids(tris: np.ndarray) -> np.ndarray:
    """The original triangle id stored in ``material_index`` by the generators."""
    return np.ascontiguousarray(tris[:, 24]).view(np.uint32)


def _face_normals(a, b, c):
    n = np.cross(b - a, c - a)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return (n / ln).astype(np.float32)


# --------------------------------------------------------------------------- #
# UV sphere (CPU configuration: 6,240 triangles)                              #
# --------------------------------------------------------------------------- #

def uv_sphere(slices: int = 80, stacks: int = 40, radius: float = 1.0, jitter: float = 0.002,
              seed: int = 0) -> np.ndarray:
    """UV sphere with pole fans; shared vertices jittered once by N(0, jitter)."""
    rng = np.random.default_rng(seed)
    theta = np.pi * np.arange(1, stacks) / stacks              # rings 1..stacks-1
    phi = 2.0 * np.pi * np.arange(slices) / slices
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    ring = np.stack([st * np.cos(phi)[None, :], np.broadcast_to(ct, (stacks - 1, slices)),
                     st * np.sin(phi)[None, :]], axis=-1) * radius   # (stacks-1, slices, 3)
    top = np.array([0.0, radius, 0.0])
    bot = np.array([0.0, -radius, 0.0])
    verts = np.concatenate([top[None], ring.reshape(-1, 3), bot[None]], axis=0)
    verts = verts + rng.normal(0.0, jitter, size=verts.shape)
    verts = verts.astype(np.float32)

    def vid(i, j):  # ring i in 1..stacks-1, slice j
        return 1 + (i - 1) * slices + (j % slices)

    tri = []
    for j in range(slices):                                   # top fan
        tri.append((0, vid(1, j), vid(1, j + 1)))
    for i in range(1, stacks - 1):                            # quads between rings
        for j in range(slices):
            v00, v10, v11, v01 = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
            tri.append((v00, v10, v11))
            tri.append((v00, v11, v01))
    last = verts.shape[0] - 1
    for j in range(slices):                                   # bottom fan
        tri.append((vid(stacks - 1, j), last, vid(stacks - 1, j + 1)))
    idx = np.asarray(tri, np.int64)
    a, b, c = verts[idx[:, 0]], verts[idx[:, 1]], verts[idx[:, 2]]
    nrm = verts / np.maximum(np.linalg.norm(verts, axis=1, keepdims=True), 1e-12)
    return _records(a, b, c, nrm[idx[:, 0]], nrm[idx[:, 1]], nrm[idx[:, 2]])


# --------------------------------------------------------------------------- #
# fBm heightfield terrain (1,048,576 triangles at 1024 x 512 quads)           #
# --------------------------------------------------------------------------- #

_M32 = np.uint64(0xFFFFFFFF)


def _hash2(ix, iz, salt):
    """Integer lattice hash -> float64 in [-1, 1)."""
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) + iz.astype(np.uint64) * np.uint64(0xD8163841)
         + np.uint64(salt) * np.uint64(0xCB1AB31F)) & _M32
    h ^= h >> np.uint64(16)
    h = (h * np.uint64(0x7FEB352D)) & _M32
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x846CA68B)) & _M32
    h ^= h >> np.uint64(16)
    return h.astype(np.float64) * (2.0 / 4294967296.0) - 1.0


def _value_noise(x, z, salt):
    ix = np.floor(x)
    iz = np.floor(z)
    fx = x - ix
    fz = z - iz
    ix = ix.astype(np.int64) & 0xFFFFFFF
    iz = iz.astype(np.int64) & 0xFFFFFFF
    sx = fx * fx * (3.0 - 2.0 * fx)
    sz = fz * fz * (3.0 - 2.0 * fz)
    v00 = _hash2(ix, iz, salt)
    v10 = _hash2(ix + 1, iz, salt)
    v01 = _hash2(ix, iz + 1, salt)
    v11 = _hash2(ix + 1, iz + 1, salt)
    a = v00 + (v10 - v00) * sx
    b = v01 + (v11 - v01) * sx
    return a + (b - a) * sz


def fbm(x, z, seed: int, octaves: int = 6, lacunarity: float = 2.0, gain: float = 0.5,
        base_freq: float = 4.0):
    total = np.zeros_like(x)
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        total += amp * _value_noise(x * freq + 17.0, z * freq + 31.0, seed * 131 + o)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return total / norm


def terrain(nx: int = 1024, nz: int = 512, height: float = 0.15, seed: int = 0) -> np.ndarray:
    """Heightfield over [-1,1]^2 with nx*nz quads, two triangles per quad."""
    xs = -1.0 + 2.0 * np.arange(nx + 1, dtype=np.float64) / nx
    zs = -1.0 + 2.0 * np.arange(nz + 1, dtype=np.float64) / nz
    X, Z = np.meshgrid(xs, zs)                                 # (nz+1, nx+1)
    Y = height * fbm(X, Z, seed)
    P = np.stack([X, Y, Z], axis=-1).astype(np.float32)
    v00 = P[:-1, :-1].reshape(-1, 3)
    v10 = P[:-1, 1:].reshape(-1, 3)
    v01 = P[1:, :-1].reshape(-1, 3)
    v11 = P[1:, 1:].reshape(-1, 3)
    a = np.stack([v00, v00], axis=1).reshape(-1, 3)
    b = np.stack([v10, v11], axis=1).reshape(-1, 3)
    c = np.stack([v11, v01], axis=1).reshape(-1, 3)
    fnrm = _face_normals(a, b, c)
    return _records(a, b, c, fnrm, fnrm, fnrm)


# --------------------------------------------------------------------------- #
# Gaussian cluster soup (4,194,304 triangles in 256 clusters)                 #
# --------------------------------------------------------------------------- #

def clusters(n_clusters: int = 256, per_cluster: int = 16384, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, size=(n_clusters, 3))
    sigma = rng.lognormal(-1.0, 0.5, size=n_clusters)
    n = n_clusters * per_cluster
    cid = np.repeat(np.arange(n_clusters), per_cluster)
    pos = centres[cid] + rng.normal(size=(n, 3)) * sigma[cid, None]
    edge = rng.lognormal(-4.0, 0.3, size=n)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    helper = np.where(np.abs(nrm[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    u = np.cross(nrm, helper)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(nrm, u)
    ang = rng.uniform(0.0, 2.0 * np.pi, size=n)
    rad = edge / math.sqrt(3.0)
    verts = []
    for k in range(3):
        th = ang + 2.0 * np.pi * k / 3.0
        verts.append(pos + rad[:, None] * (np.cos(th)[:, None] * u + np.sin(th)[:, None] * v))
    a, b, c = (x.astype(np.float32) for x in verts)
    nn = nrm.astype(np.float32)
    return _records(a, b, c, nn, nn, nn)


# --------------------------------------------------------------------------- #
# rays                                                                        #
# --------------------------------------------------------------------------- #

def tan_half_fovy(fovy_deg: float) -> np.float32:
    """The value setup_shirley_rays computes per thread (cuda-kernels.cu:63-64):
    tanf(M_PI * (fovy/2) / 180.0f), evaluated once on the host."""
    half = np.float32(fovy_deg) / np.float32(2.0)
    arg = np.float32(math.pi * float(half) / 180.0)
    return np.float32(np.tan(arg, dtype=np.float32))


class Camera:
    """Pinhole camera in the reference's Shirley setup (librta/raytrav.h:301-351)."""

    def __init__(self, pos, look_at, up=(0.0, 1.0, 0.0), fovy=60.0, w=1920, h=1080):
        self.pos = np.asarray(pos, np.float32)
        self.dir = (np.asarray(look_at, np.float32) - self.pos).astype(np.float32)
        self.up = np.asarray(up, np.float32)
        self.fovy = float(fovy)
        self.w, self.h = int(w), int(h)
        self.aspect = np.float32(np.float32(self.w) / np.float32(self.h))
        self.tan_half = tan_half_fovy(self.fovy)


def sphere_camera(w=256, h=256):
    return Camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), fovy=60.0, w=w, h=h)


def terrain_camera(w=1920, h=1080):
    return Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=w, h=h)


def incoherent_rays(n: int, extent: float = 12.0, seed: int = 0):
    """Origins uniform in [-extent, extent]^3, directions uniform on the sphere."""
    rng = np.random.default_rng(seed + 7919)
    orig = rng.uniform(-extent, extent, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    maxt = np.full(n, FLT_MAX, np.float32)
    return orig.reshape(-1), d.astype(np.float32).reshape(-1), maxt


# --------------------------------------------------------------------------- #
# batched multi-mesh workload                                                 #
# --------------------------------------------------------------------------- #

class MeshSpec:
    """One mesh of a batch: its kind, triangle count, camera and ray split."""

    def __init__(self, kind, n_tris, seed, n_rays, cam, n_primary):
        self.kind, self.n_tris, self.seed = kind, n_tris, seed
        self.n_rays, self.cam, self.n_primary = n_rays, cam, n_primary


def _lognormal_counts(rng, count, lo, hi, target_total, sigma):
    """`count` lognormal sizes clipped to [lo, hi] whose sum is close to
    target_total (the median is found by bisection on the same draws)."""
    z = rng.normal(size=count)
    a, b = math.log(lo), math.log(hi)
    for _ in range(60):
        mu = 0.5 * (a + b)
        tot = np.clip(np.exp(mu + sigma * z), lo, hi).astype(np.int64).sum()
        if tot < target_total:
            a = mu
        else:
            b = mu
    return np.clip(np.exp(0.5 * (a + b) + sigma * z), lo, hi).astype(np.int64)


def batch_specs(meshes: int = 512, seed: int = 0, total_tris: int = 25_000_000,
                tri_range=(1000, 200_000), total_rays: int = 50_000_000, ray_range=(4096, 1 << 20)):
    """The batched workload: `meshes` independent meshes, each a terrain
    (heightfield with fBm height, like the 1M-triangle terrain) or a cluster
    soup (Gaussian clusters, like the 4M-triangle one), chosen by a coin flip;
    triangle counts lognormal clipped to tri_range with a sum near total_tris;
    per-mesh ray counts lognormal clipped to ray_range with a sum near
    total_rays, half of them primary rays of a per-mesh pinhole camera, the
    rest incoherent (origins uniform in the mesh box grown by 20 %, directions
    uniform on the sphere)."""
    rng = np.random.default_rng(seed + 104729)
    nt = _lognormal_counts(rng, meshes, tri_range[0], tri_range[1], total_tris, 1.0)
    nr = _lognormal_counts(rng, meshes, ray_range[0], ray_range[1], total_rays, 1.0)
    kinds = np.where(rng.uniform(size=meshes) < 0.5, "terrain", "clusters")
    out = []
    for m in range(meshes):
        half = int(nr[m]) // 2
        h = max(1, int(math.sqrt(half * 9.0 / 16.0)))
        w = max(1, half // h)
        if kinds[m] == "terrain":
            cam = Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), fovy=60.0, w=w, h=h)
        else:
            cam = Camera((0.0, 4.0, 30.0), (0.0, 0.0, 0.0), fovy=60.0, w=w, h=h)
        out.append(MeshSpec(str(kinds[m]), int(nt[m]), seed * 100003 + m, int(nr[m]), cam, w * h))
    return out


def batch_mesh_triangles(spec: MeshSpec) -> np.ndarray:
    """The triangles of one batch mesh (104-byte records), exactly n_tris."""
    n = spec.n_tris
    if spec.kind == "terrain":
        nz = max(1, int(math.sqrt(n / 4.0)))
        nx = max(1, -(-n // (2 * nz)))
        t = terrain(nx, nz, seed=spec.seed)
    else:
        k = max(1, min(256, n // 64))
        t = clusters(k, -(-n // k), seed=spec.seed)
    return np.ascontiguousarray(t[:n])


def batch_incoherent_rays(spec: MeshSpec, tris: np.ndarray):
    """The incoherent half of a mesh's rays."""
    n = spec.n_rays - spec.n_primary
    rng = np.random.default_rng(spec.seed + 7919)
    p = tris[:, 0:9].reshape(-1, 3)
    lo, hi = p.min(0), p.max(0)
    c, e = 0.5 * (lo + hi), 0.6 * (hi - lo)
    orig = (c + rng.uniform(-1.0, 1.0, size=(n, 3)) * e).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return orig.reshape(-1), d.astype(np.float32).reshape(-1), np.full(n, FLT_MAX, np.float32)
