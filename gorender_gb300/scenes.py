"""Seeded synthetic scenes for the frame pipeline (host side, numpy only).

Every generator is deterministic across machines and numpy versions: random
numbers come from splitmix64 implemented with numpy uint64 arithmetic, and the
only transcendental functions (sin/cos for the UV sphere) are evaluated by a
fixed Taylor series with IEEE +,-,*,/ so x86 and Arm hosts produce identical
float32 meshes.

A mesh is a ``MeshData``: the arrays a ``Mesh`` (mesh.go:20-26) holds, in the
device layout the C-ABI uploads (float4 positions/normals, int32 index
triples, per-face corner UVs, per-face texture slots).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Tuple

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """splitmix64 stream (Steele, Lea & Flood 2014), vectorised."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.count = 0

    def next_u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            idx = np.arange(self.count + 1, self.count + n + 1, dtype=np.uint64)
            z = self.state + idx * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        self.count += n
        return z

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """float32 values lo + (hi-lo)*u with u a 24-bit fraction in [0,1)."""
        u = (self.next_u64(n) >> np.uint64(40)).astype(np.float64) * (1.0 / 16777216.0)
        return (lo + (hi - lo) * u).astype(np.float32)

    def integers(self, n: int, lo: int, hi: int) -> np.ndarray:
        """Integers in [lo, hi)."""
        span = np.uint64(hi - lo)
        return (self.next_u64(n) % span).astype(np.int64) + lo

    def normal(self, n: int, sigma: float = 1.0) -> np.ndarray:
        """Approximate N(0, sigma^2) as the Irwin-Hall sum of 12 uniforms - 6."""
        u = self.uniform(12 * n).astype(np.float64).reshape(n, 12)
        s = u[:, 0]
        for k in range(1, 12):
            s = s + u[:, k]
        return ((s - 6.0) * sigma).astype(np.float32)


def _det_sin_cos(x: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """sin and cos of float64 angles by a fixed Taylor series (deterministic)."""
    x = np.asarray(x, dtype=np.float64)
    two_pi = 6.283185307179586
    k = np.floor(x / two_pi + 0.5)
    r = x - k * two_pi
    r2 = r * r
    s = np.zeros_like(r)
    c = np.zeros_like(r)
    term_s = r.copy()
    term_c = np.ones_like(r)
    for n in range(0, 30):
        s = s + term_s
        c = c + term_c
        term_s = term_s * (-r2) / ((2 * n + 2) * (2 * n + 3))
        term_c = term_c * (-r2) / ((2 * n + 1) * (2 * n + 2))
    return s, c


@dataclasses.dataclass
class MeshData:
    """Arrays of one Mesh (mesh.go:20-26) in the upload layout."""

    pos: np.ndarray                      # (nv, 4) float32, w = 1
    vidx: np.ndarray                     # (nf, 3) int32
    vnrm: Optional[np.ndarray] = None    # (nn, 4) float32, w = 1
    nidx: Optional[np.ndarray] = None    # (nf, 3) int32
    uv: Optional[np.ndarray] = None      # (nf, 6) float32 corner UVs
    tex: Optional[np.ndarray] = None     # (nf,) int32 texture slot, -1 = nil
    vcolor: Optional[np.ndarray] = None  # (nv, 3) float32 RGB (extension)
    name: str = ""

    @property
    def nv(self) -> int:
        return int(self.pos.shape[0])

    @property
    def nf(self) -> int:
        return int(self.vidx.shape[0])

    def face_normals(self) -> np.ndarray:
        """NewMesh face normals (mesh.go:55-60): normalize((v1-v0)x(v2-v0)), w=1."""
        p = self.pos
        v0 = p[self.vidx[:, 0], :3]
        v1 = p[self.vidx[:, 1], :3]
        v2 = p[self.vidx[:, 2], :3]
        a = v1 - v0
        b = v2 - v0
        nx = a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1]
        ny = a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2]
        nz = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
        ln = np.sqrt(nx * nx + ny * ny + nz * nz)
        out = np.empty((self.nf, 4), dtype=np.float32)
        with np.errstate(divide="ignore", invalid="ignore"):
            out[:, 0] = nx / ln
            out[:, 1] = ny / ln
            out[:, 2] = nz / ln
        out[:, 3] = 1.0
        return out

    def bounding_box(self) -> np.ndarray:
        """boundingBox (mesh.go:28-51): 8 corners with w = 1."""
        p = self.pos
        mn = p[:, :3].min(axis=0)
        mx = p[:, :3].max(axis=0)
        (x0, y0, z0), (x1, y1, z1) = mn, mx
        return np.array([[x0, y0, z0, 1], [x0, y0, z1, 1], [x0, y1, z0, 1], [x0, y1, z1, 1],
                         [x1, y0, z0, 1], [x1, y0, z1, 1], [x1, y1, z0, 1], [x1, y1, z1, 1]],
                        dtype=np.float32)


@dataclasses.dataclass
class TextureData:
    """A Texture (texture.go:19-26).  kind: 0 solid, 1 image, 2 image-fast."""

    kind: int
    width: int = 0
    height: int = 0
    scale: float = 1.0
    color: Tuple[int, int, int, int] = (255, 0, 255, 255)
    pixels: Optional[np.ndarray] = None  # (h, w, 4) uint8

    @staticmethod
    def image(pixels: np.ndarray, scale: float = 1.0) -> "TextureData":
        h, w = pixels.shape[:2]
        pow2 = (w & (w - 1)) == 0 and (h & (h - 1)) == 0 and w > 0 and h > 0
        return TextureData(kind=2 if pow2 else 1, width=w, height=h, scale=scale,
                           pixels=np.ascontiguousarray(pixels, dtype=np.uint8))

    @staticmethod
    def solid(rgba: Tuple[int, int, int, int]) -> "TextureData":
        return TextureData(kind=0, color=tuple(int(c) for c in rgba))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def uv_sphere(lon: int = 32, lat: int = 16, radius: float = 1.0, normals: bool = True) -> MeshData:
    """UV sphere with poles: lon*(lat-2)*2 + 2*lon triangles (960 for 32x16).

    Faces are wound like the OBJ files the reference reads (counter-clockwise
    seen from outside), and vertex normals equal the unit positions.
    """
    theta = np.array([math.pi * i / lat for i in range(1, lat)], dtype=np.float64)
    phi = np.array([2.0 * math.pi * j / lon for j in range(lon)], dtype=np.float64)
    st, ct = _det_sin_cos(theta)
    sp, cp = _det_sin_cos(phi)
    ring = np.empty((lat - 1, lon, 3), dtype=np.float64)
    ring[:, :, 0] = st[:, None] * cp[None, :]
    ring[:, :, 1] = ct[:, None] * np.ones((1, lon))
    ring[:, :, 2] = -st[:, None] * sp[None, :]
    unit = np.concatenate([[[0.0, 1.0, 0.0]], ring.reshape(-1, 3), [[0.0, -1.0, 0.0]]])
    nv = unit.shape[0]
    pos = np.ones((nv, 4), dtype=np.float32)
    pos[:, :3] = (unit * radius).astype(np.float32)
    faces = []

    def rv(i, j):  # ring i (0-based), column j
        return 1 + i * lon + (j % lon)

    south = nv - 1
    for j in range(lon):
        faces.append((0, rv(0, j), rv(0, j + 1)))
    for i in range(lat - 2):
        for j in range(lon):
            a, b = rv(i, j), rv(i, j + 1)
            c, d = rv(i + 1, j), rv(i + 1, j + 1)
            faces.append((a, c, d))
            faces.append((a, d, b))
    for j in range(lon):
        faces.append((south, rv(lat - 2, j + 1), rv(lat - 2, j)))
    vidx = np.array(faces, dtype=np.int32)
    m = MeshData(pos=pos, vidx=vidx, name=f"uvsphere{lon}x{lat}")
    if normals:
        vn = np.ones((nv, 4), dtype=np.float32)
        vn[:, :3] = unit.astype(np.float32)
        m.vnrm = vn
        m.nidx = vidx.copy()
    return m


def heightfield(n: int = 317, extent: float = 4.0, amp: float = 0.1, seed: int = 0,
                uv: bool = True) -> MeshData:
    """n x n grid over [-extent, extent]^2 in x/z with heights U[-amp, amp].

    2*(n-1)^2 triangles (199,712 for n = 317), wound to face +y, with corner
    UVs (i/(n-1), j/(n-1)) so a texture scale of 8 tiles the texture 8 times.
    """
    rng = SplitMix64(seed)
    h = rng.uniform(n * n, -amp, amp).reshape(n, n)
    step = (2.0 * extent) / (n - 1)
    coords = (-extent + step * np.arange(n, dtype=np.float64)).astype(np.float32)
    pos = np.ones((n * n, 4), dtype=np.float32)
    # vertex (i, j): x = coords[i], z = coords[j]
    pos[:, 0] = np.repeat(coords, n)
    pos[:, 1] = h.reshape(-1)
    pos[:, 2] = np.tile(coords, n)
    ii, jj = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    ii = ii.reshape(-1)
    jj = jj.reshape(-1)
    a = ii * n + jj
    b = (ii + 1) * n + jj
    c = ii * n + (jj + 1)
    d = (ii + 1) * n + (jj + 1)
    t1 = np.stack([a, c, b], axis=1)
    t2 = np.stack([b, c, d], axis=1)
    vidx = np.empty((2 * a.shape[0], 3), dtype=np.int32)
    vidx[0::2] = t1
    vidx[1::2] = t2
    m = MeshData(pos=pos, vidx=vidx, name=f"heightfield{n}")
    if uv:
        inv = np.float32(1.0 / (n - 1))
        uu = (np.arange(n, dtype=np.float32) * inv).astype(np.float32)
        vi = vidx.astype(np.int64)
        gi = vi // n
        gj = vi % n
        uvs = np.empty((vidx.shape[0], 6), dtype=np.float32)
        uvs[:, 0::2] = uu[gi]
        uvs[:, 1::2] = uu[gj]
        m.uv = uvs
    return m


def icosphere(level: int, radius: float = 1.0, noise: float = 0.0, seed: int = 0,
              normals: bool = True) -> MeshData:
    """Subdivided icosahedron: 20*4^level triangles, unit normals as vn.

    ``noise`` scales each vertex radially by 1 + U[-noise, noise].
    """
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
             (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, dtype=np.float64)
    v = v / np.sqrt((v * v)[:, 0] + (v * v)[:, 1] + (v * v)[:, 2])[:, None]
    f = np.array(faces, dtype=np.int64)
    for _ in range(level):
        nvv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e_sorted = np.sort(e, axis=1)
        key = e_sorted[:, 0] * (nvv + 1) + e_sorted[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (nvv + 1)
        b = uniq % (nvv + 1)
        mid = v[a] + v[b]
        mid = mid / np.sqrt(mid[:, 0] * mid[:, 0] + mid[:, 1] * mid[:, 1] + mid[:, 2] * mid[:, 2])[:, None]
        v = np.concatenate([v, mid], axis=0)
        nf = f.shape[0]
        m01 = nvv + inv[0:nf]
        m12 = nvv + inv[nf:2 * nf]
        m20 = nvv + inv[2 * nf:3 * nf]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], axis=1),
            np.stack([f[:, 1], m12, m01], axis=1),
            np.stack([f[:, 2], m20, m12], axis=1),
            np.stack([m01, m12, m20], axis=1)], axis=0)
    unit = v
    r = np.full(unit.shape[0], radius, dtype=np.float64)
    if noise:
        r = r * (1.0 + SplitMix64(seed).uniform(unit.shape[0], -noise, noise).astype(np.float64))
    pos = np.ones((unit.shape[0], 4), dtype=np.float32)
    pos[:, :3] = (unit * r[:, None]).astype(np.float32)
    m = MeshData(pos=pos, vidx=f.astype(np.int32), name=f"icosphere{level}")
    if normals:
        vn = np.ones((unit.shape[0], 4), dtype=np.float32)
        vn[:, :3] = unit.astype(np.float32)
        m.vnrm = vn
        m.nidx = m.vidx.copy()
    return m


def random_texture(w: int = 16, h: int = 16, seed: int = 0, scale: float = 1.0) -> TextureData:
    """Random RGBA8 texture with alpha 255 (premultiplication is a no-op)."""
    rng = SplitMix64(seed)
    px = (rng.next_u64(w * h * 3) & np.uint64(0xFF)).astype(np.uint8).reshape(h, w, 3)
    rgba = np.concatenate([px, np.full((h, w, 1), 255, dtype=np.uint8)], axis=2)
    return TextureData.image(rgba, scale=scale)


@dataclasses.dataclass
class ObjectData:
    """An Object (mesh.go:71-79): mesh + scale/rotation(radians)/translation."""

    mesh: MeshData
    scale: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    rotation: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    translation: Tuple[float, float, float] = (0.0, 0.0, 0.0)


@dataclasses.dataclass
class CameraData:
    """Camera (renderer.go:22-26)."""

    position: Tuple[float, float, float] = (0.0, 0.0, 5.0)
    direction: Tuple[float, float, float] = (0.0, 0.0, -1.0)
    up: Tuple[float, float, float] = (0.0, 1.0, 0.0)


@dataclasses.dataclass
class SceneData:
    name: str
    width: int
    height: int
    objects: List[ObjectData]
    camera: CameraData
    textures: List[TextureData]
    flags: int
    fov_deg: float = 60.0

    @property
    def num_triangles(self) -> int:
        """Scene.NumTriangles (scene.go:48-54): submitted faces."""
        return sum(o.mesh.nf for o in self.objects)


# Renderer flag bits (renderer.go:90-98); the same values as the C-ABI.
FRUSTUM_CLIPPING = 0x01
SHOW_FACES = 0x02
BACKFACE_CULLING = 0x04
LIGHTING = 0x08
FLAT_SHADING = 0x10
SHOW_TEXTURES = 0x20
SHOW_EDGES = 0x40
SHOW_VERTICES = 0x80
DEFAULT_FLAGS = FRUSTUM_CLIPPING | SHOW_FACES | BACKFACE_CULLING | LIGHTING | SHOW_TEXTURES


def scene_uvsphere_640x360() -> SceneData:
    """UV sphere 32x16 (960 triangles), r = 1, Gouraud, no texture, 640x360,
    camera at (0,0,3) looking along -z, 60 degree vertical field of view."""
    m = uv_sphere(32, 16)
    return SceneData("uvsphere960-640x360", 640, 360, [ObjectData(m)],
                     CameraData((0.0, 0.0, 3.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0)), [],
                     DEFAULT_FLAGS)


def scene_heightfield_1280x720(n: int = 317) -> SceneData:
    """Heightfield 317x317 (199,712 triangles), heights U[-0.1,0.1] seed 0,
    perspective-textured with a seeded 16x16 RGBA8 texture tiled 8x, flat
    shading, 1280x720.  The camera stands inside the mesh's x/z extent, so
    triangles cross the near plane and the side planes."""
    m = heightfield(n, seed=0)
    tex = random_texture(16, 16, seed=1, scale=8.0)
    m.tex = np.zeros(m.nf, dtype=np.int32)
    cam = CameraData((0.3, 0.35, 2.5), (0.0, -0.3, -1.0), (0.0, 1.0, 0.0))
    return SceneData(f"heightfield{m.nf}-1280x720", 1280, 720, [ObjectData(m)], cam, [tex],
                     DEFAULT_FLAGS | FLAT_SHADING)


def scene_icospheres_1920x1080(count: int = 64, seed: int = 0, levels=(5, 6),
                               total_faces: Optional[int] = None) -> SceneData:
    """Small-triangle stress: ``count`` icospheres of level 5 or 6 placed
    uniformly in a 40-unit cube with scale U[0.2, 2], per-vertex RGB colours
    U[0,1] (extension), Gouraud shading, 1920x1080.

    The configuration asks for about 5 M faces in all: a level-5 sphere has
    20,480 faces and a level-6 one 81,920, so an even mix of 64 would give
    3.3 M.  With ``total_faces`` (5,000,000 by default for levels 5 and 6)
    and two levels, the number of higher-level spheres is the one whose total
    is nearest to it (60 of 64: 4,997,120 faces) and a seeded permutation
    picks which; otherwise (the smaller test scenes) each level is drawn at
    random."""
    if total_faces is None and tuple(levels) == (5, 6):
        total_faces = 5_000_000
    rng = SplitMix64(seed)
    lv = rng.integers(count, 0, len(levels))
    if total_faces is not None and len(levels) == 2:
        f_lo, f_hi = 20 * 4 ** levels[0], 20 * 4 ** levels[1]
        n_hi = int(min(count, max(0, round((total_faces - count * f_lo) / (f_hi - f_lo)))))
        order = np.argsort(SplitMix64(seed * 1000 + 7).uniform(count), kind="stable")
        lv = np.zeros(count, np.int64)
        lv[order[:n_hi]] = 1
    meshes = {}
    objs = []
    for k in range(count):
        level = levels[int(lv[k])]
        if level not in meshes:
            meshes[level] = icosphere(level)
        base = meshes[level]
        col = SplitMix64(seed * 1000 + 17 + k).uniform(base.nv * 3).reshape(base.nv, 3)
        mesh = dataclasses.replace(base, vcolor=col)
        p = rng.uniform(3, -20.0, 20.0)
        s = float(rng.uniform(1, 0.2, 2.0)[0])
        objs.append(ObjectData(mesh, scale=(s, s, s), translation=(float(p[0]), float(p[1]), float(p[2]) - 30.0)))
    cam = CameraData((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    return SceneData(f"icospheres{count}-1920x1080", 1920, 1080, objs, cam, [], DEFAULT_FLAGS)


@dataclasses.dataclass
class ViewSpec:
    """One view of a multi-view batch: its scene (objects, camera, size, flags)."""

    scene: SceneData


def multiview_batch(count: int = 256, seed: int = 0, min_tris: int = 100, max_tris: int = 200_000,
                    resolutions=((256, 256), (512, 512), (640, 360), (1280, 720))) -> List[SceneData]:
    """Views with their own mesh each: triangle counts log-uniform in
    [min_tris, max_tris] (heightfields and icospheres alternate), camera on a
    sphere of radius U[2.5, 6] looking at the origin, resolution drawn from
    ``resolutions``, material cycling through flat, Gouraud and
    perspective-textured (seeded 16x16 RGBA8)."""
    rng = SplitMix64(seed)
    out = []
    logs = rng.uniform(count, math.log(min_tris), math.log(max_tris)).astype(np.float64)
    radii = rng.uniform(count, 2.5, 6.0).astype(np.float64)
    dirs = rng.uniform(3 * count, -1.0, 1.0).astype(np.float64).reshape(count, 3)
    res_idx = rng.integers(count, 0, len(resolutions))
    for k in range(count):
        target = int(round(math.exp(logs[k])))
        material = k % 3  # 0 flat, 1 Gouraud, 2 textured
        if k % 2 == 0:
            n = max(3, int(round(math.sqrt(target / 2.0))) + 1)
            m = heightfield(n, extent=1.5, amp=0.1, seed=seed * 7919 + k, uv=(material == 2))
            if material == 1:
                # smooth-ish vertex normals pointing up for Gouraud lighting
                vn = np.zeros((m.nv, 4), np.float32)
                vn[:, 1] = 1.0
                vn[:, 3] = 1.0
                m.vnrm = vn
                m.nidx = m.vidx.copy()
        else:
            level = int(min(6, max(1, round(math.log(max(target, 20) / 20.0, 4)))))
            m = icosphere(level, noise=0.05, seed=seed * 7919 + k, normals=(material == 1))
            if material == 2:
                # spherical corner UVs
                p = m.pos[m.vidx.reshape(-1), :3].astype(np.float64)
                u = (np.arctan2(p[:, 2], p[:, 0]) / (2 * math.pi) + 0.5).astype(np.float32)
                v = (p[:, 1] * 0.5 + 0.5).astype(np.float32)
                m.uv = np.stack([u, v], axis=1).reshape(-1, 6).astype(np.float32)
        textures = []
        if material == 2:
            textures = [random_texture(16, 16, seed=seed * 31 + k, scale=4.0)]
            m.tex = np.zeros(m.nf, dtype=np.int32)
        d = dirs[k]
        nrm = math.sqrt(float((d * d).sum())) or 1.0
        pos = tuple(float(x) for x in (d / nrm * radii[k]))
        cam = CameraData(pos, tuple(-x for x in pos), (0.0, 1.0, 0.0) if abs(d[1] / nrm) < 0.95 else (1.0, 0.0, 0.0))
        w, h = resolutions[int(res_idx[k])]
        flags = DEFAULT_FLAGS | (FLAT_SHADING if material == 0 else 0)
        out.append(SceneData(f"view{k}", w, h, [ObjectData(m)], cam, textures, flags))
    return out


@dataclasses.dataclass
class DiffSceneData:
    """One mesh seen from several cameras, with the parameters of the
    differentiable shading model and a perturbed copy that renders the target."""

    mesh: MeshData
    cameras: List[CameraData]
    width: int
    height: int
    vcol: np.ndarray       # nv x 3
    tex: np.ndarray        # th x tw x 4
    light: np.ndarray      # 3
    target_params: dict    # pos, vcol, tex, light perturbed by N(0, sigma)
    flags: int = FRUSTUM_CLIPPING | SHOW_FACES | BACKFACE_CULLING
    fov_deg: float = 60.0

    @property
    def num_views(self) -> int:
        return len(self.cameras)


def spherical_uvs(m: MeshData) -> np.ndarray:
    """Per-corner UVs from the direction of each corner (u from the azimuth, v from the height)."""
    p = m.pos[m.vidx.reshape(-1), :3].astype(np.float64)
    u = (np.arctan2(p[:, 2], p[:, 0]) / (2 * math.pi) + 0.5).astype(np.float32)
    v = (p[:, 1] / np.sqrt((p * p).sum(axis=1)) * 0.5 + 0.5).astype(np.float32)
    return np.stack([u, v], axis=1).reshape(-1, 6).astype(np.float32)


def diff_scene(views: int = 64, size: int = 512, level: int = 6, tex_size: int = 256, seed: int = 0,
               sigma: float = 0.05, radius: float = 3.0) -> DiffSceneData:
    """The differentiable forward+backward workload: an icosphere (20 * 4^level
    faces) with +-5% radial noise, vertex normals, spherical UVs, vertex RGB in
    U[0,1], a tex_size^2 RGBA fp32 texture in U[0,1] and the reference's light
    direction; cameras on a sphere of the given radius looking at the origin.
    The target parameters add N(0, sigma) to positions, colours, texels and
    the light."""
    rng = SplitMix64(seed)
    m = icosphere(level, noise=0.05, seed=seed, normals=True)
    m.uv = spherical_uvs(m)
    cams = []
    d = rng.normal(3 * views).astype(np.float64).reshape(views, 3)
    for k in range(views):
        n = math.sqrt(float((d[k] * d[k]).sum())) or 1.0
        pos = tuple(float(x) for x in (d[k] / n * radius))
        up = (0.0, 1.0, 0.0) if abs(d[k][1] / n) < 0.95 else (1.0, 0.0, 0.0)
        cams.append(CameraData(pos, tuple(-x for x in pos), up))
    vcol = rng.uniform(3 * m.nv).astype(np.float32).reshape(m.nv, 3)
    tex = rng.uniform(4 * tex_size * tex_size).astype(np.float32).reshape(tex_size, tex_size, 4)
    light = np.array([-1.0, 1.0, 1.0], np.float64)
    light = (light / math.sqrt(3.0)).astype(np.float32)
    pos_t = m.pos.copy()
    pos_t[:, :3] += rng.normal(3 * m.nv, sigma).astype(np.float32).reshape(m.nv, 3)
    target = {"pos": pos_t,
              "vcol": (vcol + rng.normal(vcol.size, sigma).astype(np.float32).reshape(vcol.shape)),
              "tex": (tex + rng.normal(tex.size, sigma).astype(np.float32).reshape(tex.shape)),
              "light": (light + rng.normal(3, sigma).astype(np.float32))}
    return DiffSceneData(m, cams, size, size, vcol, tex, light, target)
