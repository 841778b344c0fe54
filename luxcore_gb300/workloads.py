"""Seeded synthetic scenes and ray batches for the LuxRays intersection path.

No public benchmark scene is named for this path, so every workload is
generated here from a seed.  Random numbers come from a counter-based
SplitMix64 stream (value i of a stream = splitmix64(key + i * golden gamma)),
which vectorises in numpy and gives the same bits on every machine.

Ray / hit layouts are luxrays::Ray (48 B) and luxrays::RayHit (20 B),
include/luxrays/core/geometry/ray_types.cl:24-36.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("d", "<f4", 3), ("mint", "<f4"), ("maxt", "<f4"),
                      ("time", "<f4"), ("flags", "<u4"), ("pad", "<f4", 2)])
HIT_DTYPE = np.dtype([("t", "<f4"), ("b1", "<f4"), ("b2", "<f4"),
                      ("meshIndex", "<u4"), ("triangleIndex", "<u4")])
assert RAY_DTYPE.itemsize == 48 and HIT_DTYPE.itemsize == 20

RAY_FLAGS_MASKED = 0x1          # ray_types.cl:22
NULL_INDEX = 0xFFFFFFFF         # luxrays_types.cl:21
BASE_SEED = 0x1D7A5EED

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _splitmix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = z + _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class Rng:
    """Counter-based SplitMix64 stream keyed by (seed, stream id)."""

    def __init__(self, seed: int, stream: int = 0):
        key = _splitmix(np.array([(seed * 0x100000001B3 + stream) & 0xFFFFFFFFFFFFFFFF],
                                 dtype=np.uint64))[0]
        self.key = np.uint64(key)
        self.counter = 0

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(self.counter, self.counter + n, dtype=np.uint64)
        self.counter += n
        with np.errstate(over="ignore"):
            return _splitmix(self.key + idx * _GAMMA)

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """float32 in [lo, hi): 24 random mantissa bits."""
        u = (self.u64(n) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))
        return (lo + (hi - lo) * u).astype(np.float32)

    def integers(self, n: int, hi: int) -> np.ndarray:
        return (self.u64(n) % np.uint64(hi)).astype(np.int64)


# ---------------------------------------------------------------------------
# scene containers
# ---------------------------------------------------------------------------

@dataclass
class Mesh:
    vertices: np.ndarray      # (nv, 3) float32
    triangles: np.ndarray     # (nt, 3) uint32, mesh-local vertex indices


@dataclass
class Motion:
    """Keyframes of a motion-blurred instance (a MotionTriangleMesh's motion
    system): strictly increasing times and (n, 4, 4) row-major matrices that
    map world space to the mesh's local space, sampled at each ray's time."""
    times: np.ndarray
    transforms: np.ndarray


@dataclass
class SceneDesc:
    """A luxrays DataSet: meshes plus ordered objects (plain or instanced).

    objects[i] = (mesh index, 4x4 row-major local-to-world matrix, a Motion,
    or None); meshIndex in a RayHit is the object's position in this list.
    """
    meshes: list
    objects: list = field(default_factory=list)

    def __post_init__(self):
        if not self.objects:
            self.objects = [(i, None) for i in range(len(self.meshes))]

    @property
    def has_instances(self) -> bool:
        return any(m is not None for _, m in self.objects)

    @property
    def has_motion(self) -> bool:
        return any(isinstance(m, Motion) for _, m in self.objects)

    def triangle_count(self) -> int:
        """Effective triangles (instances counted once per instance)."""
        return sum(int(self.meshes[mi].triangles.shape[0]) for mi, _ in self.objects)


def make_rays(o: np.ndarray, d: np.ndarray, mint, maxt, time=0.0, flags=0) -> np.ndarray:
    n = o.shape[0]
    r = np.zeros(n, dtype=RAY_DTYPE)
    r["o"] = o
    r["d"] = d
    r["mint"] = mint
    r["maxt"] = maxt
    r["time"] = time
    r["flags"] = flags
    return r


def uniform_sphere(rng: Rng, n: int) -> np.ndarray:
    z = rng.uniform(n, -1.0, 1.0).astype(np.float64)
    phi = rng.uniform(n, 0.0, 2.0 * math.pi).astype(np.float64)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1).astype(np.float32)


# ---------------------------------------------------------------------------
# Config 1 / 4 style: random small triangles in a cube
# ---------------------------------------------------------------------------

def random_triangles(n_tris: int, seed: int, extent: float = 1.0, size: float = 0.01) -> Mesh:
    """Centroids ~ U[0,extent]^3, each vertex = centroid + U[-size,size]^3."""
    rng = Rng(seed, 1)
    c = rng.uniform(3 * n_tris, 0.0, extent).reshape(n_tris, 1, 3)
    off = rng.uniform(9 * n_tris, -size, size).reshape(n_tris, 3, 3)
    v = (c + off).astype(np.float32).reshape(-1, 3)
    t = np.arange(3 * n_tris, dtype=np.uint32).reshape(n_tris, 3)
    return Mesh(v, t)


def random_triangles_fast(n_tris: int, seed: int, extent: float = 1.0, size: float = 0.01) -> Mesh:
    """random_triangles' distribution drawn with numpy's PCG64 (seeded) for
    scenes of tens of millions of triangles (serving workload)."""
    g = np.random.default_rng(seed)
    c = g.random((n_tris, 1, 3), dtype=np.float32) * np.float32(extent)
    off = (g.random((n_tris, 3, 3), dtype=np.float32) * np.float32(2 * size) - np.float32(size))
    v = (c + off).reshape(-1, 3)
    t = np.arange(3 * n_tris, dtype=np.uint32).reshape(n_tris, 3)
    return Mesh(v, t)


def random_rays(n_rays: int, seed: int, extent: float = 1.0, mint: float = 1e-4,
                maxt: float = 1e30, stream: int = 2) -> np.ndarray:
    """Origins ~ U[0,extent]^3, directions uniform on the unit sphere."""
    rng = Rng(seed, stream)
    o = rng.uniform(3 * n_rays, 0.0, extent).reshape(n_rays, 3)
    d = uniform_sphere(rng, n_rays)
    return make_rays(o, d, mint, maxt)


def config1(n_tris: int = 65536, n_rays: int = 1 << 20, seed: int = BASE_SEED + 0):
    """65,536 small random triangles in [0,1]^3 and 1,048,576 incoherent rays."""
    return SceneDesc([random_triangles(n_tris, seed)]), random_rays(n_rays, seed)


# ---------------------------------------------------------------------------
# Config 2: fBm heightfield
# ---------------------------------------------------------------------------

def _lattice(ix, iy, octave, seed):
    with np.errstate(over="ignore"):
        k = (ix.astype(np.uint64) * np.uint64(0x8CB92BA72F3D8DD7)
             ^ iy.astype(np.uint64) * np.uint64(0xD6E8FEB86659FD93)
             ^ np.uint64((seed * 1000003 + octave * 7919) & 0xFFFFFFFFFFFFFFFF))
    return (_splitmix(k) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))


def value_noise_2d(x, y, octave, seed):
    x0 = np.floor(x)
    y0 = np.floor(y)
    fx = x - x0
    fy = y - y0
    sx = fx * fx * (3.0 - 2.0 * fx)
    sy = fy * fy * (3.0 - 2.0 * fy)
    ix = x0.astype(np.int64)
    iy = y0.astype(np.int64)
    v00 = _lattice(ix, iy, octave, seed)
    v10 = _lattice(ix + 1, iy, octave, seed)
    v01 = _lattice(ix, iy + 1, octave, seed)
    v11 = _lattice(ix + 1, iy + 1, octave, seed)
    a = v00 + (v10 - v00) * sx
    b = v01 + (v11 - v01) * sx
    return a + (b - a) * sy


def fbm_heights(res: int, seed: int, octaves: int = 6, base_freq: float = 4.0,
                lacunarity: float = 2.0, gain: float = 0.5, hmax: float = 0.2) -> np.ndarray:
    g = np.linspace(0.0, 1.0, res, dtype=np.float64)
    x, y = np.meshgrid(g, g, indexing="xy")
    h = np.zeros_like(x)
    amp, freq = 1.0, base_freq
    for o in range(octaves):
        h += amp * value_noise_2d(x * freq, y * freq, o, seed)
        amp *= gain
        freq *= lacunarity
    h = (h - h.min()) / max(h.max() - h.min(), 1e-30) * hmax
    return h.astype(np.float32)


def heightfield_mesh(res: int = 1024, seed: int = BASE_SEED + 1) -> Mesh:
    """res x res vertex grid over [0,1]^2, 2*(res-1)^2 triangles."""
    h = fbm_heights(res, seed)
    g = np.linspace(0.0, 1.0, res, dtype=np.float32)
    x, y = np.meshgrid(g, g, indexing="xy")
    v = np.stack([x, y, h], axis=-1).reshape(-1, 3).astype(np.float32)
    i = np.arange(res - 1, dtype=np.uint32)
    ii, jj = np.meshgrid(i, i, indexing="xy")
    v00 = (jj * res + ii).ravel()
    v10 = v00 + 1
    v01 = v00 + res
    v11 = v01 + 1
    t = np.concatenate([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], axis=0)
    # interleave the two triangles of each cell so triangle order follows the grid
    t = t.reshape(2, -1, 3).transpose(1, 0, 2).reshape(-1, 3)
    return Mesh(v, t.astype(np.uint32))


def pinhole_rays(width: int, height: int, eye=(0.5, -0.5, 0.6), look=(0.5, 0.5, 0.0),
                 up=(0.0, 0.0, 1.0), fov_deg: float = 60.0, mint: float = 1e-4,
                 maxt: float = 1e30) -> np.ndarray:
    eye = np.array(eye, np.float64)
    fwd = np.array(look, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.array(up, np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    tan_half = math.tan(math.radians(fov_deg) * 0.5)
    aspect = width / height
    px = (np.arange(width) + 0.5) / width * 2.0 - 1.0
    py = 1.0 - (np.arange(height) + 0.5) / height * 2.0
    X, Y = np.meshgrid(px * tan_half * aspect, py * tan_half, indexing="xy")
    d = fwd[None, :] + X.reshape(-1, 1) * right[None, :] + Y.reshape(-1, 1) * upv[None, :]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(eye, d.shape)
    return make_rays(o.astype(np.float32), d.astype(np.float32), mint, maxt)


def geometric_normals(scene: SceneDesc, hits: np.ndarray) -> np.ndarray:
    """Unit geometric normal of each hit triangle (plain objects only)."""
    n = np.zeros((hits.shape[0], 3), np.float64)
    for oi, (mi, m) in enumerate(scene.objects):
        sel = np.nonzero(hits["meshIndex"] == oi)[0]
        if sel.size == 0:
            continue
        mesh = scene.meshes[mi]
        tri = mesh.triangles[hits["triangleIndex"][sel]]
        p0 = mesh.vertices[tri[:, 0]].astype(np.float64)
        p1 = mesh.vertices[tri[:, 1]].astype(np.float64)
        p2 = mesh.vertices[tri[:, 2]].astype(np.float64)
        nn = np.cross(p1 - p0, p2 - p0)
        if m is not None:
            inv_t = np.linalg.inv(np.asarray(m, np.float64).reshape(4, 4))[:3, :3]
            nn = nn @ inv_t
        n[sel] = nn / np.maximum(np.linalg.norm(nn, axis=1, keepdims=True), 1e-30)
    return n


def bounce_rays(scene: SceneDesc, rays: np.ndarray, hits: np.ndarray, n_out: int,
                seed: int, mint: float = 1e-4, maxt: float = 1e30) -> np.ndarray:
    """Cosine-hemisphere rays about the geometric normal at hit points
    (hit points cycled when there are fewer hits than n_out)."""
    hit_idx = np.nonzero(hits["meshIndex"] != NULL_INDEX)[0]
    if hit_idx.size == 0:
        raise ValueError("no primary hits to bounce from")
    src = hit_idx[np.arange(n_out) % hit_idx.size]
    o = rays["o"][src].astype(np.float64) + rays["d"][src].astype(np.float64) * hits["t"][src, None]
    nrm = geometric_normals(scene, hits[src])
    flip = np.sum(nrm * rays["d"][src], axis=1) > 0
    nrm[flip] *= -1.0
    rng = Rng(seed, 5)
    u1 = rng.uniform(n_out).astype(np.float64)
    u2 = rng.uniform(n_out).astype(np.float64)
    r = np.sqrt(u1)
    phi = 2.0 * math.pi * u2
    lx, ly, lz = r * np.cos(phi), r * np.sin(phi), np.sqrt(np.maximum(0.0, 1.0 - u1))
    a = np.where(np.abs(nrm[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(nrm, a)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(nrm, t)
    d = t * lx[:, None] + b * ly[:, None] + nrm * lz[:, None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return make_rays(o.astype(np.float32), d.astype(np.float32), mint, maxt)


def shadow_rays(origins_rays: np.ndarray, n_lights: int, seed: int, mint: float = 1e-4) -> np.ndarray:
    """Rays from each origin to n_lights point lights ~ U[0,1]^2 x [0.5,1]."""
    rng = Rng(seed, 6)
    lights = np.stack([rng.uniform(n_lights), rng.uniform(n_lights),
                       rng.uniform(n_lights, 0.5, 1.0)], axis=1).astype(np.float64)
    o = np.repeat(origins_rays["o"].astype(np.float64), n_lights, axis=0)
    L = np.tile(lights, (origins_rays.shape[0], 1))
    d = L - o
    dist = np.linalg.norm(d, axis=1)
    d /= np.maximum(dist[:, None], 1e-30)
    return make_rays(o.astype(np.float32), d.astype(np.float32), mint,
                     (dist * (1.0 - 1e-4)).astype(np.float32))


# ---------------------------------------------------------------------------
# Config 3: instanced displaced icospheres
# ---------------------------------------------------------------------------

_PHI = (1.0 + 5 ** 0.5) / 2.0
_ICO_V = np.array([[-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
                   [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
                   [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]], np.float64)
_ICO_F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                   [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                   [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                   [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)


def value_noise_3d(p: np.ndarray, seed: int, freq: float = 4.0) -> np.ndarray:
    q = p * freq
    i0 = np.floor(q)
    f = q - i0
    s = f * f * (3.0 - 2.0 * f)
    ii = i0.astype(np.int64)
    acc = 0.0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                with np.errstate(over="ignore"):
                    k = ((ii[:, 0] + dx).astype(np.uint64) * np.uint64(0x8CB92BA72F3D8DD7)
                         ^ (ii[:, 1] + dy).astype(np.uint64) * np.uint64(0xD6E8FEB86659FD93)
                         ^ (ii[:, 2] + dz).astype(np.uint64) * np.uint64(0xA0761D6478BD642F)
                         ^ np.uint64(seed & 0xFFFFFFFFFFFFFFFF))
                v = (_splitmix(k) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))
                w = ((s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1])
                     * (s[:, 2] if dz else 1 - s[:, 2]))
                acc = acc + w * v
    return acc


def displaced_icosphere(freq: int, seed: int, disp: float = 0.2) -> Mesh:
    """Geodesic icosphere (20*freq^2 faces) with a radial displacement in
    [0, disp] from 3D value noise; vertices are per icosahedron face."""
    a, b = np.meshgrid(np.arange(freq + 1), np.arange(freq + 1), indexing="ij")
    keep = (a + b) <= freq
    a, b = a[keep], b[keep]                      # barycentric lattice of one face
    nloc = a.size
    lut = -np.ones((freq + 1, freq + 1), np.int64)
    lut[a, b] = np.arange(nloc)
    tris = []
    for i in range(freq):
        for j in range(freq - i):
            tris.append((lut[i, j], lut[i + 1, j], lut[i, j + 1]))
            if i + j + 1 < freq:
                tris.append((lut[i + 1, j], lut[i + 1, j + 1], lut[i, j + 1]))
    tris = np.array(tris, np.int64)              # freq^2 triangles per face
    verts, faces = [], []
    for fi, (ia, ib, ic) in enumerate(_ICO_F):
        A, B, C = _ICO_V[ia], _ICO_V[ib], _ICO_V[ic]
        p = (A[None] * (freq - a - b)[:, None] + B[None] * a[:, None] + C[None] * b[:, None]) / freq
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        verts.append(p)
        faces.append(tris + fi * nloc)
    v = np.concatenate(verts, 0)
    r = 1.0 + disp * value_noise_3d(v, seed)
    v = v * r[:, None]
    return Mesh(v.astype(np.float32), np.concatenate(faces, 0).astype(np.uint32))


def random_rotation(rng: Rng, n: int) -> np.ndarray:
    """Uniform random rotations (Shoemake's unit quaternions) as 3x3 matrices."""
    u1, u2, u3 = (rng.uniform(n).astype(np.float64) for _ in range(3))
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * math.pi * u2), np.sqrt(1 - u1) * np.cos(2 * math.pi * u2),
                  np.sqrt(u1) * np.sin(2 * math.pi * u3), np.sqrt(u1) * np.cos(2 * math.pi * u3)], 1)
    x, y, z, w = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], 1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], 1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1)], 1)


def instanced_scene(n_meshes: int = 16, freq: int = 100, n_inst: int = 4096,
                    seed: int = BASE_SEED + 2, scale=(0.01, 0.05), extent: float = 10.0) -> SceneDesc:
    meshes = [displaced_icosphere(freq, seed * 31 + k) for k in range(n_meshes)]
    rng = Rng(seed, 7)
    rot = random_rotation(rng, n_inst)
    s = rng.uniform(n_inst, scale[0], scale[1]).astype(np.float64)
    tr = rng.uniform(3 * n_inst, 0.0, extent).reshape(n_inst, 3).astype(np.float64)
    mids = rng.integers(n_inst, n_meshes)
    objects = []
    for k in range(n_inst):
        m = np.eye(4, dtype=np.float64)
        m[:3, :3] = rot[k] * s[k]
        m[:3, 3] = tr[k]
        objects.append((int(mids[k]), m.astype(np.float32)))
    return SceneDesc(meshes, objects)


def config3(n_rays: int = 1 << 23, seed: int = BASE_SEED + 2, **kw):
    scene = instanced_scene(seed=seed, **kw)
    ext = kw.get("extent", 10.0)
    closest = random_rays(n_rays, seed, extent=ext, stream=8)
    anyhit = random_rays(n_rays, seed, extent=ext, stream=9)
    anyhit["maxt"] = Rng(seed, 10).uniform(n_rays, 0.5, 5.0)
    return scene, closest, anyhit


def motion_scene(n_meshes: int = 16, freq: int = 100, n_inst: int = 4096, seed: int = BASE_SEED + 4,
                 scale=(0.01, 0.05), extent: float = 10.0, kinds=("translate", "rigid", "static"),
                 speed: float = 0.003) -> SceneDesc:
    """instanced_scene with motion blur: instance k becomes a Motion of kind
    kinds[k % len(kinds)] over the shutter [0, 1] --
      "translate": two keyframes moving by up to `speed` * extent per axis
                   (about an instance's size at the defaults; the
                   world->local matrices differ in translation only);
      "rigid":     three keyframes (times 0, 0.5, 1) turning about a random
                   axis by up to 90 degrees, scaling by up to 1.5x and moving;
      "static":    a plain instance (its local->world matrix).
    Keyframes are world->local: the float64 inverse of the local->world
    matrix at that time, rounded to float32."""
    base = instanced_scene(n_meshes, freq, n_inst, seed, scale, extent)
    rng = Rng(seed, 12)
    cz = rng.uniform(n_inst, -1.0, 1.0).astype(np.float64)
    az = rng.uniform(n_inst, 0.0, 2.0 * math.pi).astype(np.float64)
    axis = np.stack([np.sqrt(1 - cz * cz) * np.cos(az), np.sqrt(1 - cz * cz) * np.sin(az), cz], 1)
    ang = rng.uniform(n_inst, 0.0, 0.5 * math.pi).astype(np.float64)
    grow = rng.uniform(n_inst, 1.0, 1.5).astype(np.float64)
    move = rng.uniform(3 * n_inst, -1.0, 1.0).reshape(n_inst, 3).astype(np.float64) * speed * extent

    def turn(k, a):
        x, y, z = axis[k]
        c, s = math.cos(a), math.sin(a)
        return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                         [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                         [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])

    objects = []
    for k, (mi, m) in enumerate(base.objects):
        kind = kinds[k % len(kinds)]
        m = m.astype(np.float64)
        if kind == "static":
            objects.append((mi, m.astype(np.float32)))
            continue
        times = [0.0, 1.0] if kind == "translate" else [0.0, 0.5, 1.0]
        keys = []
        for t in times:
            lw = m.copy()
            if kind == "rigid":
                lw[:3, :3] = turn(k, ang[k] * t) @ m[:3, :3] * (1.0 + (grow[k] - 1.0) * t)
            lw[:3, 3] = m[:3, 3] + move[k] * t
            keys.append(np.linalg.inv(lw))
        objects.append((mi, Motion(np.asarray(times, np.float32), np.stack(keys).astype(np.float32))))
    return SceneDesc(base.meshes, objects)


def config_motion(n_rays: int = 1 << 23, seed: int = BASE_SEED + 4, time_range=(0.0, 1.0), **kw):
    """Motion-blurred instances (motion_scene) with closest-hit and any-hit
    rays whose times are uniform over `time_range`."""
    scene = motion_scene(seed=seed, **kw)
    ext = kw.get("extent", 10.0)
    closest = random_rays(n_rays, seed, extent=ext, stream=13)
    anyhit = random_rays(n_rays, seed, extent=ext, stream=14)
    anyhit["maxt"] = Rng(seed, 15).uniform(n_rays, 0.5, 5.0)
    closest["time"] = Rng(seed, 16).uniform(n_rays, *time_range)
    anyhit["time"] = Rng(seed, 17).uniform(n_rays, *time_range)
    return scene, closest, anyhit


# ---------------------------------------------------------------------------
# Config 4: uneven batches over several resident scenes
# ---------------------------------------------------------------------------

def log_uniform_int(rng: Rng, n: int, lo: int, hi: int) -> np.ndarray:
    u = rng.uniform(n).astype(np.float64)
    return np.floor(np.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))).astype(np.int64)


def uneven_batches(n_scenes: int = 8, n_batches: int = 512, tri_range=(100_000, 4_000_000),
                   size_range=(1024, 2_097_152), anyhit_frac: float = 0.3,
                   seed: int = BASE_SEED + 3):
    """Scene triangle counts, batch sizes, scene choice and mode per batch.
    Returns (tri_counts, extents, [(scene, size, anyhit)])."""
    rng = Rng(seed, 11)
    tri_counts = log_uniform_int(rng, n_scenes, *tri_range)
    extents = (tri_counts / 65536.0) ** (1.0 / 3.0)
    sizes = log_uniform_int(rng, n_batches, *size_range)
    scenes = rng.integers(n_batches, n_scenes)
    anyhit = rng.uniform(n_batches) < anyhit_frac
    return tri_counts, extents, list(zip(scenes.tolist(), sizes.tolist(), anyhit.tolist()))
