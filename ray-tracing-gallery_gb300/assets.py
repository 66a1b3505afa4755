"""Asset files for the ray-tracing core.

Decoding goes through librtcore.so (include/rtassets.h, host code, no GPU
needed); the scene assembly mirrors the reference's start-up code:

=================================  ==============================================
this module                        reference (src/...)
=================================  ==============================================
decode_png                         util_functions.rs:239-265 load_png_image_from_bytes
load_glb                           util_structs.rs:1049-1156 Model::load_gltf
TextureTable.push_image            util_structs.rs:1338-1358 ImageManager::push_image
default_scene                      main.rs:416-459 (fixed images), scene.rs:35-159
                                   DefaultScene::new, main.rs:568-598 (camera, sun)
default_scene_instances            scene.rs:163-204 (update, write_resources)
first_person_view_inverse          main.rs:1206-1231 FirstPersonCamera
=================================  ==============================================

The reference draws the 100 small tori of its default scene from an unseeded
`thread_rng` (scene.rs:136); here they come from PCG32(seed), drawn in the
same order (x, y, z, rotation, scale, shader).

The reference's asset files are not part of this package.  `standin_assets`
writes files of the same kinds and sizes from seeds (PNG and GLB writers
below): a 2-triangle plane, two linked tori of 2,304 triangles, a 45,448-triangle
textured figure with a linearly filtered texture, an alpha-masked
double-sided fence, 1x1 RGB fallback colours, a 16-bit grey 64x64 blue-noise
image and an RGBA8 lookup table.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import struct
import zlib

import numpy as np

from . import abi
from .scenes import Geometry, Model, Pcg32, Scene, Texture, affine, instance_records, make_uniforms, \
    perspective_reversed_infinite_z_vk_inverse, rot_y


def _lib():
    return abi.load_library()


def decode_png(data: bytes) -> np.ndarray:
    """PNG bytes -> (H, W, 4) uint8 RGBA (`to_rgba8` of the decoded image)."""
    lib = _lib()
    buf = C.create_string_buffer(bytes(data), len(data))
    w, h = C.c_uint32(), C.c_uint32()
    abi.check(lib, lib.rt_png_decode_rgba8(buf, len(data), None, 0, C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value, 4), np.uint8)
    abi.check(lib, lib.rt_png_decode_rgba8(buf, len(data), out.ctypes.data, out.nbytes, C.byref(w), C.byref(h)))
    return out


class TextureTable(dict):
    """The bindless image array: index -> Texture, filled in push order."""

    def push_image(self, tex: Texture) -> int:
        idx = len(self)
        self[idx] = tex
        return idx


def read_glb(data: bytes) -> dict:
    """Decodes a GLB file: vertex arrays, per-geometry indices / flags /
    model image slots, and the model's images in push order."""
    lib = _lib()
    buf = C.create_string_buffer(bytes(data), len(data))
    handle = C.c_void_p()
    abi.check(lib, lib.rt_glb_load(buf, len(data), C.byref(handle)))
    try:
        info = abi.RtGlbInfo()
        abi.check(lib, lib.rt_glb_info(handle, C.byref(info)))
        v = info.vertex_count
        pos = np.empty((v, 3), np.float32)
        nrm = np.empty((v, 3), np.float32)
        uv = np.empty((v, 2), np.float32)
        abi.check(lib, lib.rt_glb_read_vertices(handle, pos.ctypes.data, nrm.ctypes.data, uv.ctypes.data))
        geoms = []
        for g in range(info.geometry_count):
            gi = abi.RtGlbGeometry()
            abi.check(lib, lib.rt_glb_read_geometry(handle, g, C.byref(gi), None, 0))
            idx = np.empty(gi.index_count, np.uint32)
            abi.check(lib, lib.rt_glb_read_geometry(handle, g, C.byref(gi), idx.ctypes.data, idx.size))
            geoms.append(dict(indices=idx.reshape(-1, 3), opaque=bool(gi.opaque), diffuse=gi.diffuse_image,
                              metallic_roughness=gi.metallic_roughness_image, normal_map=gi.normal_map_image))
        images = []
        for i in range(info.image_count):
            ii = abi.RtGlbImage()
            abi.check(lib, lib.rt_glb_read_image(handle, i, C.byref(ii), None, 0))
            if ii.format == abi.RT_FORMAT_R32G32B32A32_SFLOAT:
                tex = np.empty((ii.height, ii.width, 4), np.float32)
            else:
                tex = np.empty((ii.height, ii.width, 4), np.uint8)
            abi.check(lib, lib.rt_glb_read_image(handle, i, C.byref(ii), tex.ctypes.data, tex.nbytes))
            images.append(Texture(tex, ii.format, ii.filter))
        return dict(positions=pos, normals=nrm, uvs=uv, geometries=geoms, images=images,
                    primitive_count=info.primitive_count, triangle_count=info.triangle_count)
    finally:
        lib.rt_glb_destroy(handle)


def load_glb(data: bytes, name: str, fallback_image_index: int, textures: TextureTable) -> Model:
    """Model::load_gltf: the model's images are pushed into `textures` in
    order; a geometry without a diffuse image takes fallback_image_index."""
    d = read_glb(data)
    slots = [textures.push_image(t) for t in d["images"]]
    geoms = []
    for g in d["geometries"]:
        geoms.append(Geometry(g["indices"], g["opaque"],
                              slots[g["diffuse"]] if g["diffuse"] >= 0 else fallback_image_index,
                              slots[g["metallic_roughness"]],
                              slots[g["normal_map"]] if g["normal_map"] >= 0 else -1))
    return Model(d["positions"], d["normals"], d["uvs"], geoms, name)


# ---------------------------------------------------------------------------
# The reference's default scene
# ---------------------------------------------------------------------------
DEFAULT_ASSETS = ("green.png", "pink.png", "blue_noise_64x64.png", "flipped_ggx_lut.png",
                  "plane.glb", "tori.glb", "lain.glb", "fence.glb")
DEFAULT_WIDTH, DEFAULT_HEIGHT = 1280, 720        # main.rs:82 window size
LAIN_BASE_ROTATION = math.radians(150.0)          # scene.rs:91
LAIN_ROTATION_STEP = 0.05                         # scene.rs:164
SMALL_TORI = 100                                  # scene.rs:138


def first_person_view_inverse(eye, pitch: float, yaw: float) -> np.ndarray:
    """Camera-to-world of FirstPersonCamera::as_view_matrix (main.rs:1208-1230):
    the view matrix's rows are the camera axes, so its inverse has them as
    columns with the eye as translation.  Column-major float32."""
    x = (math.cos(yaw), 0.0, -math.sin(yaw))
    y = (math.sin(yaw) * math.sin(pitch), math.cos(pitch), math.cos(yaw) * math.sin(pitch))
    z = (math.sin(yaw) * math.cos(pitch), -math.sin(pitch), math.cos(pitch) * math.cos(yaw))
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = x, y, z, eye
    return m.T.reshape(-1).astype(np.float32)


def sun_normal(pitch: float, yaw: float) -> tuple[float, float, float]:
    """Sun::as_normal (main.rs:1189-1197)."""
    return (math.cos(pitch) * math.sin(yaw), math.sin(pitch), math.cos(pitch) * math.cos(yaw))


def default_scene_transforms(seed: int = 0, frame: int = 0):
    """Instance transforms, model ids, hit shaders and double-sided flags of
    DefaultScene::new (scene.rs:94-155); instance 2 (the figure) turned by
    frame * 0.05 rad (scene.rs:163-165)."""
    H = (abi.HIT_SHADER_TEXTURED, abi.HIT_SHADER_MIRROR, abi.HIT_SHADER_PORTAL)
    xf, mdl, sbt, ds = [], [], [], []

    def add(t, m, s, d):
        xf.append(t); mdl.append(m); sbt.append(s); ds.append(d)

    add(affine(np.eye(3), [0, 0, 0], 10.0), 0, H[0], False)
    add(affine(np.eye(3), [0, 1, 0]), 1, H[0], False)
    add(affine(rot_y(LAIN_BASE_ROTATION + LAIN_ROTATION_STEP * frame), [-2, 0, -1], 0.5), 2, H[0], False)
    add(affine(np.eye(3), [0, 1, 0]), 0, H[2], True)
    add(affine(np.eye(3), [2, 0, 2]), 3, H[0], True)
    rng = Pcg32(seed, 0xDEFA)
    for _ in range(SMALL_TORI):
        t = [rng.uniform_range(-10.0, 10.0), rng.uniform_range(0.5, 2.5), rng.uniform_range(-10.0, 10.0)]
        r = rot_y(rng.uniform_range(0.0, 100.0))
        s = rng.uniform_range(0.01, 0.1)
        add(affine(r, t, s), 1, H[0] if rng.next_u32() & 1 else H[1], False)
    return np.array(xf), np.array(mdl), np.array(sbt), np.array(ds)


def default_scene_instances(seed: int = 0, frame: int = 0) -> np.ndarray:
    """Instance records (BLAS = model id; custom index = model id, mask 0xFF,
    gpu_structs.rs:28-52) of the default scene at `frame`."""
    xf, mdl, sbt, ds = default_scene_transforms(seed, frame)
    flags = np.where(ds, abi.RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE, 0)
    return instance_records(xf, mdl, mdl, sbt, flags)


def default_scene_uniforms(width: int, height: int, frame: int = 0) -> abi.RtUniforms:
    """main.rs:568-598: camera at (0, 2, -5), pitch 0, yaw 180 deg; sun pitch
    0.5, yaw 1.0, radius 0.05; 59 deg vertical field of view, near 0.1;
    blue noise image 2, GGX LUT image 3."""
    return make_uniforms(first_person_view_inverse((0.0, 2.0, -5.0), 0.0, math.radians(180.0)),
                         perspective_reversed_infinite_z_vk_inverse(math.radians(59.0), width / height, 0.1),
                         sun_normal(0.5, 1.0), 0.05, 2, 3, frame)


def default_scene(assets: dict[str, bytes], width: int = DEFAULT_WIDTH, height: int = DEFAULT_HEIGHT,
                  seed: int = 0, frame: int = 1) -> Scene:
    """The reference's default scene from its asset files: images 0-3 are
    green, pink (sRGB, nearest), blue noise (UNORM, nearest) and the GGX LUT
    (UNORM, linear); then the plane (fallback image 0), tori (1), figure (1)
    and fence (0) models push their own images; 105 instances; 3 bounce
    iterations and 2 shadow rays (closest_hit_textured.glsl:195)."""
    tex = TextureTable()
    tex.push_image(Texture(decode_png(assets["green.png"]), abi.RT_FORMAT_R8G8B8A8_SRGB))
    tex.push_image(Texture(decode_png(assets["pink.png"]), abi.RT_FORMAT_R8G8B8A8_SRGB))
    tex.push_image(Texture(decode_png(assets["blue_noise_64x64.png"]), abi.RT_FORMAT_R8G8B8A8_UNORM))
    tex.push_image(Texture(decode_png(assets["flipped_ggx_lut.png"]), abi.RT_FORMAT_R8G8B8A8_UNORM,
                           abi.RT_FILTER_LINEAR))
    models = [load_glb(assets["plane.glb"], "plane", 0, tex), load_glb(assets["tori.glb"], "tori", 1, tex),
              load_glb(assets["lain.glb"], "lain", 1, tex), load_glb(assets["fence.glb"], "fence", 0, tex)]
    if len(tex) > abi.RT_MAX_BOUND_IMAGES:
        raise ValueError(f"{len(tex)} images exceed the bound-image limit {abi.RT_MAX_BOUND_IMAGES}")
    return Scene(models, dict(tex), default_scene_instances(seed, frame), default_scene_uniforms(width, height, frame),
                 width, height, max_trace_depth=3, shadow_ray_count=2, name="default-scene",
                 extra={"seed": seed, "frame": frame})


# ---------------------------------------------------------------------------
# Writers for synthetic asset files
# ---------------------------------------------------------------------------
def _png_chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _pack_rows(samples: np.ndarray, depth: int) -> np.ndarray:
    """(h, w*channels) integer samples -> (h, rowbytes) uint8, big-endian,
    sub-byte samples packed from the most significant bit."""
    h, n = samples.shape
    if depth == 16:
        s = samples.astype(">u2")
        return s.view(np.uint8).reshape(h, n * 2)
    if depth == 8:
        return samples.astype(np.uint8)
    per = 8 // depth
    pad = (-n) % per
    s = np.concatenate([samples.astype(np.uint8), np.zeros((h, pad), np.uint8)], 1).reshape(h, -1, per)
    out = np.zeros(s.shape[:2], np.uint8)
    for k in range(per):
        out |= (s[:, :, k] << (8 - depth * (k + 1))).astype(np.uint8)
    return out


def _filter_rows(rows: np.ndarray, bpp: int, filters) -> bytes:
    """Applies PNG row filters (type filters[y % len]) to unfiltered rows."""
    h, n = rows.shape
    r = rows.astype(np.int32)
    out = bytearray()
    prev = np.zeros(n, np.int32)
    for y in range(h):
        x = r[y]
        a = np.concatenate([np.zeros(bpp, np.int32), x[:-bpp]]) if n > bpp else np.zeros(n, np.int32)
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]]) if n > bpp else np.zeros(n, np.int32)
        b = prev
        ft = filters[y % len(filters)]
        if ft == 0:
            f = x
        elif ft == 1:
            f = x - a
        elif ft == 2:
            f = x - b
        elif ft == 3:
            f = x - (a + b) // 2
        else:
            p = a + b - c
            pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
            f = x - np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        out.append(ft)
        out += (f & 0xFF).astype(np.uint8).tobytes()
        prev = x
    return bytes(out)


def encode_png(samples: np.ndarray, color_type: int, depth: int = 8, interlace: bool = False,
               filters=(0, 1, 2, 3, 4), palette: np.ndarray | None = None, trns: bytes | None = None,
               level: int = 6, idat_split: int = 0, extra_chunks: tuple = ()) -> bytes:
    """Encodes (H, W, channels) integer samples as a PNG of the given colour
    type and bit depth (row filters cycled through `filters`)."""
    s = np.asarray(samples)
    if s.ndim == 2:
        s = s[:, :, None]
    h, w, ch = s.shape
    assert ch == _CHANNELS[color_type]
    bits_pp = ch * depth
    bpp = max(1, bits_pp // 8)
    raw = b""
    passes = _ADAM7 if interlace else ((0, 0, 1, 1),)
    for x0, y0, dx, dy in passes:
        sub = s[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        rows = _pack_rows(sub.reshape(sub.shape[0], -1), depth)
        raw += _filter_rows(rows, bpp, filters)
    z = zlib.compress(raw, level)
    out = b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color_type, 0, 0,
                                                                   1 if interlace else 0))
    for kind, data in extra_chunks:
        out += _png_chunk(kind, data)
    if palette is not None:
        out += _png_chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += _png_chunk(b"tRNS", trns)
    step = idat_split or len(z)
    for i in range(0, len(z), step):
        out += _png_chunk(b"IDAT", z[i:i + step])
    return out + _png_chunk(b"IEND", b"")


def encode_glb(doc: dict, binary: bytes) -> bytes:
    """glTF 2.0 binary container: header, JSON chunk (space padded), BIN
    chunk (zero padded)."""
    js = json.dumps(doc, separators=(",", ":")).encode()
    js += b" " * ((-len(js)) % 4)
    bn = bytes(binary) + b"\0" * ((-len(binary)) % 4)
    body = struct.pack("<II", len(js), 0x4E4F534A) + js
    if bn:
        body += struct.pack("<II", len(bn), 0x004E4942) + bn
    return struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body


class GlbBuilder:
    """Accumulates buffer views / accessors / meshes / materials / images for
    encode_glb."""

    def __init__(self):
        self.bin = bytearray()
        self.doc = {"asset": {"version": "2.0", "generator": "rtgallery stand-in writer"},
                    "buffers": [{"byteLength": 0}], "bufferViews": [], "accessors": [], "meshes": [],
                    "nodes": [], "scenes": [{"nodes": []}], "scene": 0}

    def view(self, data: bytes, stride: int = 0) -> int:
        while len(self.bin) % 4:
            self.bin.append(0)
        v = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)}
        if stride:
            v["byteStride"] = stride
        self.bin += data
        self.doc["bufferViews"].append(v)
        return len(self.doc["bufferViews"]) - 1

    def accessor(self, arr: np.ndarray, kind: str, ctype: int, normalized: bool = False) -> int:
        a = {"bufferView": self.view(np.ascontiguousarray(arr).tobytes()), "componentType": ctype,
             "count": int(arr.shape[0]), "type": kind}
        if normalized:
            a["normalized"] = True
        if kind == "VEC3" and ctype == 5126:
            a["min"] = [float(x) for x in arr.min(0)]
            a["max"] = [float(x) for x in arr.max(0)]
        self.doc["accessors"].append(a)
        return len(self.doc["accessors"]) - 1

    def image(self, png: bytes, mag_filter: int | None = 9729) -> int:
        d = self.doc
        d.setdefault("images", []).append({"bufferView": self.view(png), "mimeType": "image/png"})
        smp = {} if mag_filter is None else {"magFilter": mag_filter}
        d.setdefault("samplers", []).append(smp)
        d.setdefault("textures", []).append({"sampler": len(d["samplers"]) - 1, "source": len(d["images"]) - 1})
        return len(d["textures"]) - 1

    def material(self, **m) -> int:
        self.doc.setdefault("materials", []).append(m)
        return len(self.doc["materials"]) - 1

    def mesh(self, positions, normals, uvs, indices, material: int | None = None, index_type: int = 5123,
             node: dict | None = None) -> int:
        idx = np.asarray(indices).reshape(-1).astype({5121: np.uint8, 5123: np.uint16, 5125: np.uint32}[index_type])
        prim = {"attributes": {"POSITION": self.accessor(np.asarray(positions, np.float32), "VEC3", 5126),
                               "NORMAL": self.accessor(np.asarray(normals, np.float32), "VEC3", 5126),
                               "TEXCOORD_0": self.accessor(np.asarray(uvs, np.float32), "VEC2", 5126)},
                "indices": self.accessor(idx, "SCALAR", index_type)}
        if material is not None:
            prim["material"] = material
        self.doc["meshes"].append({"primitives": [prim]})
        n = dict(node or {})
        n["mesh"] = len(self.doc["meshes"]) - 1
        self.doc["nodes"].append(n)
        self.doc["scenes"][0]["nodes"].append(len(self.doc["nodes"]) - 1)
        return n["mesh"]

    def encode(self) -> bytes:
        self.doc["buffers"][0]["byteLength"] = len(self.bin)
        return encode_glb(self.doc, bytes(self.bin))


def _lathe(profile_r: np.ndarray, profile_y: np.ndarray, segments: int):
    """Surface of revolution about +Y: (len(profile)-1) * segments quads."""
    nv = len(profile_r) - 1
    u = np.arange(segments + 1) / segments
    v = np.arange(nv + 1) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    phi = 2 * np.pi * U
    r = profile_r[None, :].repeat(segments + 1, 0)
    y = profile_y[None, :].repeat(segments + 1, 0)
    pos = np.stack([r * np.cos(phi), y, r * np.sin(phi)], -1).reshape(-1, 3)
    # normals from the profile's slope
    dr = np.gradient(profile_r)
    dy = np.gradient(profile_y)
    n2 = np.stack([dy, -dr], -1)
    n2 /= np.maximum(np.linalg.norm(n2, axis=1, keepdims=True), 1e-12)
    nr = n2[None, :, 0].repeat(segments + 1, 0)
    ny = n2[None, :, 1].repeat(segments + 1, 0)
    nrm = np.stack([nr * np.cos(phi), ny, nr * np.sin(phi)], -1).reshape(-1, 3)
    uv = np.stack([U, 1.0 - V], -1).reshape(-1, 2)
    i, j = np.meshgrid(np.arange(segments), np.arange(nv), indexing="ij")
    a = i * (nv + 1) + j
    b = (i + 1) * (nv + 1) + j
    tris = np.stack([np.stack([a, a + 1, b + 1], -1), np.stack([a, b + 1, b], -1)], 2).reshape(-1, 3)
    return pos.astype(np.float32), nrm.astype(np.float32), uv.astype(np.float32), tris.astype(np.uint32)


def _quad(width: float, height: float, vertical: bool):
    if vertical:   # in the XY plane, facing -Z
        pos = [[-width / 2, 0, 0], [width / 2, 0, 0], [width / 2, height, 0], [-width / 2, height, 0]]
        nrm = [[0, 0, -1]] * 4
    else:          # in the XZ plane, facing +Y
        pos = [[-width / 2, 0, -height / 2], [width / 2, 0, -height / 2], [width / 2, 0, height / 2],
               [-width / 2, 0, height / 2]]
        nrm = [[0, 1, 0]] * 4
    uv = [[0, 1], [1, 1], [1, 0], [0, 0]]
    idx = [[0, 2, 1], [0, 3, 2]] if not vertical else [[0, 1, 2], [0, 2, 3]]
    return (np.array(pos, np.float32), np.array(nrm, np.float32), np.array(uv, np.float32),
            np.array(idx, np.uint32))


def standin_assets(seed: int = 0, figure_texture: int = 512) -> dict[str, bytes]:
    """Synthetic files with the names, kinds and sizes of the reference's
    default-scene assets (see the module docstring)."""
    from .scenes import torus

    rng = np.random.default_rng(seed)
    out = {}
    out["green.png"] = encode_png(np.array([[[40, 200, 60]]], np.uint8), 2)
    out["pink.png"] = encode_png(np.array([[[235, 120, 190]]], np.uint8), 2)
    ranks = rng.permutation(64 * 64).reshape(64, 64)
    out["blue_noise_64x64.png"] = encode_png((ranks * 65535 // 4095).astype(np.uint16), 0, 16)
    yy, xx = np.mgrid[0:256, 0:256] / 255.0
    lut = np.stack([xx * 255, yy * 255, (1 - xx * yy) * 255, np.full_like(xx, 255)], -1).astype(np.uint8)
    out["flipped_ggx_lut.png"] = encode_png(lut, 6)

    b = GlbBuilder()
    b.mesh(*_quad(2.0, 2.0, vertical=False), node={"scale": [10, 10, 10]})   # node scale is not applied
    out["plane.glb"] = b.encode()

    # two linked tori of 1,152 triangles each in one primitive: 2,304 triangles
    b = GlbBuilder()
    p0, n0, u0, i0 = torus(1.0, 0.25, 32, 18)
    p1 = (p0 @ np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], np.float32).T) + np.float32([1.0, 0, 0])
    n1 = n0 @ np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], np.float32).T
    b.mesh(np.concatenate([p0, p1]), np.concatenate([n0, n1]), np.concatenate([u0, u0]),
           np.concatenate([i0, i0 + len(p0)]))
    out["tori.glb"] = b.encode()

    # figure: a lathe body, 247 segments x 92 profile steps = 45,448 triangles
    t = np.linspace(0.0, 1.0, 93)
    prof_y = 4.8 * t
    prof_r = 0.05 + 0.6 * np.sin(np.pi * t) ** 0.7 * (0.75 + 0.25 * np.cos(6 * np.pi * t))
    b = GlbBuilder()
    n = figure_texture
    ty, tx = np.mgrid[0:n, 0:n]
    body = np.stack([120 + 100 * np.sin(tx * 0.05), 90 + 60 * np.cos(ty * 0.07), 150 + 80 * np.sin((tx + ty) * 0.03),
                     np.full((n, n), 255.0)], -1)
    body += rng.integers(-12, 13, body.shape)
    tex = b.image(encode_png(np.clip(body, 0, 255).astype(np.uint8), 6), 9729)
    mat = b.material(doubleSided=True, pbrMetallicRoughness={"baseColorTexture": {"index": tex},
                                                              "metallicFactor": 0, "roughnessFactor": 0.5})
    b.mesh(*_lathe(prof_r, prof_y, 247), material=mat)
    out["lain.glb"] = b.encode()

    # fence: alpha-masked double-sided quad (alpha holes in a lattice)
    b = GlbBuilder()
    fy, fx = np.mgrid[0:256, 0:256]
    bars = ((fx % 32) < 6) | ((fy % 32) < 6)
    ftex = np.stack([np.full((256, 256), 150), np.full((256, 256), 110), np.full((256, 256), 70),
                     np.where(bars, 255, 0)], -1).astype(np.uint8)
    tex = b.image(encode_png(ftex, 6), 9729)
    mat = b.material(alphaMode="MASK", alphaCutoff=0.5, doubleSided=True,
                     pbrMetallicRoughness={"baseColorTexture": {"index": tex}, "metallicFactor": 0,
                                           "roughnessFactor": 0.5})
    b.mesh(*_quad(2.0, 2.0, vertical=True), material=mat)
    out["fence.glb"] = b.encode()
    return out
