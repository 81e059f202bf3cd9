"""Host-side loaders feeding the device upload: Wavefront OBJ/MTL meshes
(obj.go:196-309), scene manifests (scene.go:56-133) and image textures
(texture.go:35-63, 91-103), restated from the reference's behaviour.

* Numbers are parsed as Go's fmt.Sscanf("%f") into a float32 does: the
  decimal text correctly rounded to float32 (not through a double).
* Faces must be triangles ("mesh is not triangulated" otherwise: exactly three
  spaces after TrimSpace) in one of the forms ``v``, ``v/vt``, ``v//vn`` or
  ``v/vt/vn``; indices are 1-based and relative to the objects read so far.
* The ``v//vn`` form reproduces obj.go:81 by default: the third normal index is
  scanned into the second slot, so the second corner gets the third normal and
  the third corner's normal index becomes ``-offset - 1`` (a bad index that the
  reference panics on when it lights with vertex normals, and that the library
  reports as GR_ERR_BAD_INDEX).  ``fix_normal_indices=True`` reads the three
  normals as written.
* ``usemtl`` picks the material's ``map_Kd`` texture (loaded once per file
  name); a material without ``map_Kd`` gets the solid magenta texture; an
  unknown material leaves faces untextured.
* Textures decode PNG (every colour type, bit depth and interlacing of the
  PNG specification) and convert each pixel as color.RGBAModel.Convert does,
  i.e. alpha-premultiplied 8-bit RGBA: for non-premultiplied input,
  out = ((c * 257 * a) // 255) >> 8 at 8 bits and ((c16 * a16) // 65535) >> 8 at
  16 bits.  Power-of-two sizes select the fast (mask) sampler.  JPEG (which
  texture.go:6 also registers) is rejected with a clear error: Go's decoder
  could not be matched bit for bit against any Go output here.
* Scene manifests: every mesh of the manifest is its file's first mesh
  (LoadMeshFile(..., true)); its faces all take the manifest's texture (with
  textureScale when non-zero) or the solid (200, 200, 200, 255) colour; object
  rotations are degrees turned into radians as Vec3.ToRadians does,
  v * float32(pi32 / 180).  JSON keys match case-insensitively, as
  encoding/json does.
"""
from __future__ import annotations

import dataclasses
import fractions
import json
import math
import os
import struct
import zlib
from typing import Dict, List, Optional, Tuple

import numpy as np

from .scenes import CameraData, DEFAULT_FLAGS, MeshData, ObjectData, SceneData, TextureData

__all__ = ["parse_float32", "load_obj", "load_texture", "decode_png", "load_scene", "LoadedScene"]


# ---------------------------------------------------------------------------
# numbers
# ---------------------------------------------------------------------------

def parse_float32(tok: str) -> np.float32:
    """strconv.ParseFloat(tok, 32): the decimal value correctly rounded to
    float32 (round half to even), without the double rounding of
    float32(float(tok))."""
    d = float(tok)
    f = np.float32(d)
    if not math.isfinite(d) or not np.isfinite(f):
        return f
    # double rounding can only go wrong when d is exactly halfway between two
    # float32 values; then the exact decimal decides
    lo = np.nextafter(f, np.float32(-np.inf)) if float(f) > d else f
    hi = np.nextafter(lo, np.float32(np.inf))
    mid = (fractions.Fraction(float(lo)) + fractions.Fraction(float(hi))) / 2
    if fractions.Fraction(d) != mid:
        return f
    x = fractions.Fraction(tok.strip().replace("_", ""))
    if x < mid:
        return lo
    if x > mid:
        return hi
    # an exact tie: the even mantissa
    return lo if (int(lo.view(np.uint32)) & 1) == 0 else hi


def _float32_deg_to_rad(v: np.float32) -> np.float32:
    """Vec3.ToRadians (vector.go:82-85): v * (pi32 / 180), pi32 = float32(math.Pi)."""
    pi32 = fractions.Fraction(float(np.float32(math.pi)))
    f = _round_fraction_f32(pi32 / 180)
    return np.float32(np.float32(v) * f)


def _round_fraction_f32(x: fractions.Fraction) -> np.float32:
    f = np.float32(float(x))
    cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
    best = min(cands, key=lambda c: (abs(fractions.Fraction(float(c)) - x), int(c.view(np.uint32)) & 1))
    return best


# ---------------------------------------------------------------------------
# PNG (decoded from the PNG specification; converted as Go's image/color does)
# ---------------------------------------------------------------------------

_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
_DEPTHS = {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}


def _unfilter(data: bytes, pos: int, width: int, height: int, bpp: int, row_bytes: int):
    """Reverses the five PNG scanline filters; returns (rows as uint8 array, new position)."""
    out = np.zeros((height, row_bytes), np.uint8)
    prev = np.zeros(row_bytes, np.int32)
    for y in range(height):
        if pos >= len(data):
            raise ValueError("png: not enough pixel data")
        ft = data[pos]
        raw = np.frombuffer(data, np.uint8, row_bytes, pos + 1).astype(np.int32)
        pos += 1 + row_bytes
        if ft == 0:
            cur = raw
        elif ft == 1:
            cur = raw.copy()
            for i in range(bpp, row_bytes):
                cur[i] = (cur[i] + cur[i - bpp]) & 0xFF
        elif ft == 2:
            cur = (raw + prev) & 0xFF
        elif ft == 3:
            cur = raw.copy()
            for i in range(row_bytes):
                left = cur[i - bpp] if i >= bpp else 0
                cur[i] = (cur[i] + ((left + prev[i]) >> 1)) & 0xFF
        elif ft == 4:
            cur = raw.copy()
            for i in range(row_bytes):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (cur[i] + pred) & 0xFF
        else:
            raise ValueError(f"png: bad filter type {ft}")
        out[y] = cur
        prev = cur
    return out, pos


def _samples(rows: np.ndarray, width: int, depth: int, channels: int) -> np.ndarray:
    """Unpacks scanlines to (h, w, channels) integer samples."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :width * channels].reshape(h, width, channels).astype(np.int64)
    if depth == 16:
        r = rows[:, :width * channels * 2].reshape(h, width * channels, 2).astype(np.int64)
        return (r[..., 0] * 256 + r[..., 1]).reshape(h, width, channels)
    bits = np.unpackbits(rows, axis=1)[:, :width * depth].reshape(h, width, depth).astype(np.int64)
    val = np.zeros((h, width), np.int64)
    for k in range(depth):
        val = val * 2 + bits[..., k]
    return val.reshape(h, width, 1)


def decode_png(data: bytes) -> np.ndarray:
    """Decodes a PNG into premultiplied RGBA8 (H x W x 4), as LoadTextureFile +
    NewImageTexture produce it (color.RGBAModel.Convert of every pixel)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("png: not a PNG file")
    pos = 8
    ihdr = None
    plte = None
    trns = None
    idat = []
    while pos + 8 <= len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if zlib.crc32(typ + body) & 0xFFFFFFFF != crc:
            raise ValueError(f"png: bad CRC in {typ!r}")
        pos += 12 + n
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3).astype(np.int64)
        elif typ == b"tRNS":
            trns = body
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
    if ihdr is None:
        raise ValueError("png: missing IHDR")
    W, H, depth, ct, comp, filt, inter = ihdr
    if ct not in _CHANNELS or depth not in _DEPTHS[ct] or comp or filt or inter > 1:
        raise ValueError(f"png: unsupported format (colour type {ct}, depth {depth}, interlace {inter})")
    ch = _CHANNELS[ct]
    raw = zlib.decompress(b"".join(idat))
    bpp = max(1, (depth * ch) // 8)
    samples = np.zeros((H, W, ch), np.int64)
    pos = 0
    passes = _ADAM7 if inter == 1 else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        pw = (W - x0 + dx - 1) // dx if W > x0 else 0
        ph = (H - y0 + dy - 1) // dy if H > y0 else 0
        if pw == 0 or ph == 0:
            continue
        row_bytes = (pw * depth * ch + 7) // 8
        rows, pos = _unfilter(raw, pos, pw, ph, bpp, row_bytes)
        samples[y0::dy, x0::dx] = _samples(rows, pw, depth, ch)
    return _to_rgba_model(samples, ct, depth, plte, trns)


def _premul8(c, a):
    # color.NRGBA.RGBA(): c16 = (c * 0x101) * a / 0xff; RGBAModel keeps c16 >> 8
    return ((c * 257 * a) // 255) >> 8


def _to_rgba_model(s: np.ndarray, ct: int, depth: int, plte, trns) -> np.ndarray:
    H, W = s.shape[:2]
    out = np.zeros((H, W, 4), np.uint8)
    if ct == 3:
        if plte is None:
            raise ValueError("png: missing palette")
        # entries past the palette read as opaque black, as Go's decoder fills them
        pal = np.zeros((256, 4), np.int64)
        pal[:, 3] = 255
        pal[:len(plte), :3] = plte
        if trns is not None:
            t = np.frombuffer(trns, np.uint8).astype(np.int64)[:len(plte)]
            pal[:len(t), 3] = t
        a = pal[:, 3]
        pm = np.stack([_premul8(pal[:, k], a) for k in range(3)] + [a], axis=1)
        return pm[s[..., 0]].astype(np.uint8)
    if depth == 16:
        # 16-bit: Gray16 / RGBA64 (opaque) or NRGBA64: c16 * a16 / 0xffff, then >> 8
        if ct in (0, 2):
            rgb = np.repeat(s, 3, axis=2) if ct == 0 else s
            a16 = np.full((H, W), 65535, np.int64)
            if trns is not None:
                key = np.frombuffer(trns, ">u2").astype(np.int64)
                match = (s[..., 0] == key[0]) if ct == 0 else (s == key[:3]).all(axis=2)
                a16 = np.where(match, 0, 65535)
        else:
            rgb = np.repeat(s[..., :1], 3, axis=2) if ct == 4 else s[..., :3]
            a16 = s[..., -1]
        for k in range(3):
            out[..., k] = ((rgb[..., k] * a16) // 65535) >> 8
        out[..., 3] = a16 >> 8
        return out
    if ct == 0:
        scale = {1: 0xFF, 2: 0x55, 4: 0x11, 8: 1}[depth]
        y = s[..., 0] * scale
        a = np.full((H, W), 255, np.int64)
        if trns is not None:
            key = struct.unpack(">H", trns[:2])[0]
            a = np.where(s[..., 0] == key, 0, 255)
        for k in range(3):
            out[..., k] = _premul8(y, a)
        out[..., 3] = a
        return out
    if ct == 2:
        a = np.full((H, W), 255, np.int64)
        if trns is not None:
            key = np.array(struct.unpack(">HHH", trns[:6]), np.int64)
            a = np.where((s == key).all(axis=2), 0, 255)
        for k in range(3):
            out[..., k] = _premul8(s[..., k], a)
        out[..., 3] = a
        return out
    if ct == 4:
        a = s[..., 1]
        for k in range(3):
            out[..., k] = _premul8(s[..., 0], a)
        out[..., 3] = a
        return out
    a = s[..., 3]
    for k in range(3):
        out[..., k] = _premul8(s[..., k], a)
    out[..., 3] = a
    return out


def load_texture(path: str, scale: float = 1.0) -> TextureData:
    """LoadTextureFile + NewImageTexture: the fast sampler for power-of-two sizes."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:3] == b"\xff\xd8\xff":
        raise ValueError(f"{path}: JPEG textures are not decoded here (convert the texture to PNG)")
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: only PNG textures are decoded here")
    return TextureData.image(decode_png(data), scale=float(np.float32(scale)))


# ---------------------------------------------------------------------------
# OBJ / MTL
# ---------------------------------------------------------------------------

MAGENTA = (255, 0, 255, 255)   # obj.go:205 default texture of a material without map_Kd
DEFAULT_COLOR = (200, 200, 200, 255)  # scene.go:75


def _parse_mtl(path: str) -> List[Tuple[str, str]]:
    """parseMtlLibFile (obj.go:152-190): (name, map_Kd) in file order."""
    mats: List[List[str]] = []
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            if line.startswith("newmtl "):
                mats.append([line[len("newmtl "):], ""])
            elif line.startswith("map_Kd "):
                if not mats:
                    raise ValueError(f"{path}: map_Kd before newmtl")  # a nil dereference in the reference
                mats[-1][1] = line[len("map_Kd "):]
    return [(n, m) for n, m in mats]


def _scan(line: str, head: str, n: int, conv):
    toks = line.split()
    if not toks or toks[0] != head or len(toks) < n + 1:
        raise ValueError(f"cannot parse {line!r}")
    return [conv(t) for t in toks[1:n + 1]]


@dataclasses.dataclass
class _Ctx:
    verts: list
    uvs: list
    normals: list
    faces: list          # (vidx[3], nidx[3], uv[6], texture key or None)
    voff: int = 0
    toff: int = 0
    noff: int = 0


def _parse_face(c: _Ctx, line: str, fix_normal_indices: bool):
    if line.count(" ") != 3:
        raise ValueError("mesh is not triangulated")
    toks = line.split(" ")[1:]
    nidx = [0, 0, 0]
    uv = [0.0] * 6
    if line.count("//") == 3:
        parts = [t.split("//") for t in toks]
        v = [int(p[0]) for p in parts]
        vn = [int(p[1]) for p in parts]
        if not fix_normal_indices:
            vn = [vn[0], vn[2], 0]  # obj.go:81 scans the third index into the second slot
        nidx = [x - c.noff - 1 for x in vn]
    elif line.count("/") == 3:
        parts = [t.split("/") for t in toks]
        v = [int(p[0]) for p in parts]
        for k, p in enumerate(parts):
            t = int(p[1]) - c.toff - 1
            if t < 0 or t >= len(c.uvs):
                raise ValueError(f"texture vertex index out of range in {line!r}")
            uv[2 * k], uv[2 * k + 1] = c.uvs[t]
    elif line.count("/") == 6:
        parts = [t.split("/") for t in toks]
        v = [int(p[0]) for p in parts]
        for k, p in enumerate(parts):
            t = int(p[1]) - c.toff - 1
            if t < 0 or t >= len(c.uvs):
                raise ValueError(f"texture vertex index out of range in {line!r}")
            uv[2 * k], uv[2 * k + 1] = c.uvs[t]
        nidx = [int(p[2]) - c.noff - 1 for p in parts]
    else:
        v = [int(t) for t in toks]
    return [x - c.voff - 1 for x in v], nidx, uv


def _finish_mesh(c: _Ctx, name: str, tex_index: Dict[int, int]) -> MeshData:
    nv = len(c.verts)
    pos = np.ones((nv, 4), np.float32)
    if nv:
        pos[:, :3] = np.array(c.verts, np.float32).reshape(nv, 3)
    vidx = np.array([f[0] for f in c.faces], np.int32).reshape(-1, 3)
    if vidx.size and (vidx.min() < 0 or vidx.max() >= nv):
        raise ValueError(f"{name}: vertex index out of range")  # NewMesh panics in the reference
    m = MeshData(pos=pos, vidx=vidx, name=name)
    if c.normals:
        vn = np.ones((len(c.normals), 4), np.float32)
        vn[:, :3] = np.array(c.normals, np.float32).reshape(-1, 3)
        m.vnrm = vn
    m.nidx = np.array([f[1] for f in c.faces], np.int32).reshape(-1, 3)
    m.uv = np.array([f[2] for f in c.faces], np.float32).reshape(-1, 6)
    tex = [tex_index.get(id(f[3]), -1) if f[3] is not None else -1 for f in c.faces]
    m.tex = np.array(tex, np.int32)
    return m


def load_obj(path: str, single_mesh: bool = False, fix_normal_indices: bool = False,
             textures: Optional[List[TextureData]] = None) -> Tuple[List[MeshData], List[TextureData]]:
    """LoadObjFile (obj.go:194-309).  Returns the meshes and the texture list
    their ``tex`` arrays index (textures are appended to ``textures`` when given)."""
    texs: List[TextureData] = textures if textures is not None else []
    tex_index: Dict[int, int] = {}
    dirname = os.path.dirname(path)
    by_name: Dict[str, Optional[TextureData]] = {}
    by_file: Dict[str, TextureData] = {}
    default = TextureData.solid(MAGENTA)
    current = None
    c = _Ctx([], [], [], [])
    meshes: List[MeshData] = []

    def register(t: TextureData):
        if id(t) not in tex_index:
            tex_index[id(t)] = len(texs)
            texs.append(t)

    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            if line.startswith("mtllib "):
                for name, map_kd in _parse_mtl(os.path.join(dirname, line[len("mtllib "):])):
                    if not map_kd:
                        by_name[name] = default
                    elif map_kd in by_file:
                        by_name[name] = by_file[map_kd]
                    else:
                        tp = map_kd if map_kd.startswith("/") else os.path.join(dirname, map_kd)
                        t = load_texture(tp)
                        by_file[map_kd] = t
                        by_name[name] = t
            elif line.startswith("o "):
                if c.verts and not single_mesh:
                    meshes.append(_finish_mesh(c, f"{os.path.basename(path)}#{len(meshes)}", tex_index))
                    c = _Ctx([], [], [], [], c.voff + len(c.verts), c.toff + len(c.uvs), c.noff + len(c.normals))
            elif line.startswith("v "):
                c.verts.append(_scan(line, "v", 3, parse_float32))
            elif line.startswith("vt "):
                c.uvs.append(_scan(line, "vt", 2, parse_float32))
            elif line.startswith("vn "):
                c.normals.append(_scan(line, "vn", 3, parse_float32))
            elif line.startswith("usemtl "):
                current = by_name.get(line[len("usemtl "):])
                if current is not None:
                    register(current)
            elif line.startswith("f "):
                vidx, nidx, uv = _parse_face(c, line, fix_normal_indices)
                c.faces.append((vidx, nidx, uv, current))
    if c.verts:
        meshes.append(_finish_mesh(c, f"{os.path.basename(path)}#{len(meshes)}", tex_index))
    if not meshes:
        raise ValueError("obj file does not have any vertices data")
    return meshes, texs


# ---------------------------------------------------------------------------
# scene manifests
# ---------------------------------------------------------------------------

def _get(d: dict, key: str, default=None):
    """encoding/json field matching: exact name first, then case-insensitive."""
    if key in d:
        return d[key]
    low = key.lower()
    for k, v in d.items():
        if k.lower() == low:
            return v
    return default


def _vec3(v) -> Tuple[np.float32, np.float32, np.float32]:
    if v is None:
        return (np.float32(0), np.float32(0), np.float32(0))
    return tuple(parse_float32(str(x)) for x in v)


@dataclasses.dataclass
class LoadedScene:
    """A loaded manifest: objects (meshes shared by id) and the texture list."""

    name: str
    objects: List[ObjectData]
    textures: List[TextureData]

    def scene(self, width: int, height: int, camera: CameraData, flags: int = DEFAULT_FLAGS,
              fov_deg: float = 60.0) -> SceneData:
        return SceneData(self.name, width, height, self.objects, camera, self.textures, flags, fov_deg)


def load_scene(path: str) -> LoadedScene:
    """LoadSceneFile (scene.go:56-133)."""
    with open(path, "r", encoding="utf-8") as f:
        data = json.load(f, parse_float=str, parse_int=str)
    root = os.path.dirname(path)
    textures: List[TextureData] = []
    default = TextureData.solid(DEFAULT_COLOR)
    meshes: Dict[str, MeshData] = {}
    for md in _get(data, "meshes", []) or []:
        mid = _get(md, "id", "")
        loaded, _ = load_obj(os.path.join(root, _get(md, "objFile", "")), single_mesh=True)
        mesh = loaded[0]
        tex_file = _get(md, "texture", "")
        if tex_file:
            t = load_texture(os.path.join(root, tex_file))
            scale = parse_float32(str(_get(md, "textureScale", "0")))
            if scale != 0:
                t = dataclasses.replace(t, scale=float(scale))
        else:
            t = default
        if not any(t is x for x in textures):
            textures.append(t)
        slot = next(i for i, x in enumerate(textures) if x is t)
        mesh = dataclasses.replace(mesh, tex=np.full(mesh.nf, slot, np.int32))
        meshes[mid] = mesh
    objects: List[ObjectData] = []
    for od in _get(data, "objects", []) or []:
        mid = _get(od, "meshID", "")
        if mid not in meshes:
            raise ValueError(f"mesh id not found: {mid}")
        rot = tuple(float(_float32_deg_to_rad(r)) for r in _vec3(_get(od, "rotation")))
        objects.append(ObjectData(meshes[mid], scale=tuple(float(x) for x in _vec3(_get(od, "scale"))),
                                  rotation=rot, translation=tuple(float(x) for x in _vec3(_get(od, "position")))))
    return LoadedScene(str(_get(data, "name", "")), objects, textures)
