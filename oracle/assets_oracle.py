"""CPU oracle for the asset decoders (TEST INFRASTRUCTURE ONLY).

A second, independent statement of what the reference's start-up code does
with its asset files, used by tests/ to check librtcore's native decoders
(include/rtassets.h).  Nothing in the product imports this module.

  png_decode_rgba8   load_png_image_from_bytes, src/util_functions.rs:239-265:
                     `image` 0.23.14 / `png` 0.16.8 decode with EXPAND, then
                     to_rgba8.  Inflate is Python's zlib (an implementation
                     independent of the library's); unfiltering and the
                     colour expansion are restated here in plain Python.
  glb_decode         Model::load_gltf, src/util_structs.rs:1049-1156, with
                     load_images_from_material :982-1024 and
                     load_image_from_gltf_texture :934-980 (`gltf` 0.16.0):
                     one geometry per material, images pushed per material
                     as diffuse, metallic-roughness, normal map.

Parity pins: the reference has no tests for these paths.  The oracle is
checked against fixtures whose expected texels are the very samples that
were encoded (tests/golden/make_asset_fixtures.py) and, in a checkout that
has the reference's resources/, against the triangle counts its glTF headers
state (2, 2,304, 45,448, 2).  The 16-bit -> 8-bit step (high byte) restates
the `image` 0.23 channel conversion and is not pinned by any reference
output.
"""
from __future__ import annotations

import json
import struct
import zlib

import numpy as np

RT_FORMAT_R8G8B8A8_UNORM = 37
RT_FORMAT_R8G8B8A8_SRGB = 43
RT_FORMAT_R32G32B32A32_SFLOAT = 109
RT_FILTER_NEAREST = 0
RT_FILTER_LINEAR = 1

_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


class DecodeError(ValueError):
    pass


def _chunks(data: bytes):
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise DecodeError("signature")
    at = 8
    while at + 12 <= len(data):
        (n,) = struct.unpack_from(">I", data, at)
        kind = data[at + 4:at + 8]
        body = data[at + 8:at + 8 + n]
        if len(body) != n or at + 12 + n > len(data):
            raise DecodeError("truncated chunk")
        (crc,) = struct.unpack_from(">I", data, at + 8 + n)
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise DecodeError("crc")
        yield kind, body
        at += 12 + n
        if kind == b"IEND":
            return
    raise DecodeError("no IEND")


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw: bytes, at: int, h: int, rowbytes: int, bpp: int) -> list[bytearray]:
    rows = []
    prev = bytearray(rowbytes)
    for _ in range(h):
        ft = raw[at]
        r = bytearray(raw[at + 1:at + 1 + rowbytes])
        at += rowbytes + 1
        if ft == 1:
            for i in range(bpp, rowbytes):
                r[i] = (r[i] + r[i - bpp]) & 0xFF
        elif ft == 2:
            for i in range(rowbytes):
                r[i] = (r[i] + prev[i]) & 0xFF
        elif ft == 3:
            for i in range(rowbytes):
                a = r[i - bpp] if i >= bpp else 0
                r[i] = (r[i] + ((a + prev[i]) >> 1)) & 0xFF
        elif ft == 4:
            for i in range(rowbytes):
                a = r[i - bpp] if i >= bpp else 0
                c = prev[i - bpp] if i >= bpp else 0
                r[i] = (r[i] + _paeth(a, prev[i], c)) & 0xFF
        elif ft != 0:
            raise DecodeError(f"filter {ft}")
        rows.append(r)
        prev = r
    return rows


def _samples(row: bytearray, count: int, depth: int) -> list[int]:
    if depth == 8:
        return list(row[:count])
    if depth == 16:
        return [row[2 * i] << 8 | row[2 * i + 1] for i in range(count)]
    per = 8 // depth
    mask = (1 << depth) - 1
    return [(row[i // per] >> (8 - depth * (i % per + 1))) & mask for i in range(count)]


def png_decode_rgba8(data: bytes) -> np.ndarray:
    """(H, W, 4) uint8, the reference's to_rgba8 of the decoded PNG."""
    hdr, plte, trns, idat = None, None, None, b""
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = body
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat += body
    if hdr is None:
        raise DecodeError("no IHDR")
    w, h, depth, color, _, _, interlace = hdr
    ch = _CHANNELS[color]
    bits_pp = ch * depth
    bpp = max(1, bits_pp // 8)
    raw = zlib.decompress(idat)
    out = np.zeros((h, w, 4), np.uint8)
    to8 = (lambda v: v >> 8) if depth == 16 else (lambda v: v) if depth == 8 else \
        (lambda v, s=255 // ((1 << depth) - 1): v * s)
    at = 0
    for x0, y0, dx, dy in (_ADAM7 if interlace else ((0, 0, 1, 1),)):
        pw = (w - x0 + dx - 1) // dx if w > x0 else 0
        ph = (h - y0 + dy - 1) // dy if h > y0 else 0
        if not pw or not ph:
            continue
        rowbytes = (pw * bits_pp + 7) // 8
        rows = _unfilter(raw, at, ph, rowbytes, bpp)
        at += ph * (rowbytes + 1)
        for j, r in enumerate(rows):
            s = _samples(r, pw * ch, depth)
            y = y0 + j * dy
            for i in range(pw):
                px = s[i * ch:(i + 1) * ch]
                x = x0 + i * dx
                if color == 0:
                    g = to8(px[0])
                    a = 0 if trns is not None and px[0] == (trns[0] << 8 | trns[1]) else 255
                    out[y, x] = (g, g, g, a)
                elif color == 2:
                    key = trns is not None and tuple(px) == tuple(trns[k] << 8 | trns[k + 1] for k in (0, 2, 4))
                    out[y, x] = (to8(px[0]), to8(px[1]), to8(px[2]), 0 if key else 255)
                elif color == 3:
                    k = px[0]
                    if 3 * k + 2 >= len(plte):
                        raise DecodeError("palette index")
                    a = trns[k] if trns is not None and k < len(trns) else 255
                    out[y, x] = (plte[3 * k], plte[3 * k + 1], plte[3 * k + 2], a)
                elif color == 4:
                    g = to8(px[0])
                    out[y, x] = (g, g, g, to8(px[1]))
                else:
                    out[y, x] = tuple(to8(v) for v in px)
    return out


_CTYPE = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}


def _accessor(doc: dict, binary: bytes, index: int) -> np.ndarray:
    a = doc["accessors"][index]
    v = doc["bufferViews"][a["bufferView"]]
    dt = np.dtype(_CTYPE[a["componentType"]]).newbyteorder("<")
    n = _NCOMP[a["type"]]
    elem = dt.itemsize * n
    stride = v.get("byteStride", elem)
    base = v.get("byteOffset", 0) + a.get("byteOffset", 0)
    rows = [np.frombuffer(binary, dt, n, base + i * stride) for i in range(a["count"])] if stride != elem else None
    if rows is None:
        arr = np.frombuffer(binary, dt, a["count"] * n, base).reshape(a["count"], n)
    else:
        arr = np.array(rows).reshape(a["count"], n)
    return arr


def glb_decode(data: bytes) -> dict:
    """Vertex arrays, geometries and images (in push order) of a GLB file."""
    magic, version, length = struct.unpack_from("<III", data, 0)
    if magic != 0x46546C67 or version != 2:
        raise DecodeError("not GLB 2")
    at, doc, binary = 12, None, b""
    while at + 8 <= length:
        n, kind = struct.unpack_from("<II", data, at)
        body = data[at + 8:at + 8 + n]
        if kind == 0x4E4F534A and doc is None:
            doc = json.loads(body)
        elif kind == 0x004E4942 and not binary:
            binary = body
        at += 8 + ((n + 3) & ~3)
    images, geoms, decoded = [], [], {}

    def texture(info, fmt):
        tex = doc["textures"][info["index"]]
        filt = RT_FILTER_LINEAR
        if "sampler" in tex and doc["samplers"][tex["sampler"]].get("magFilter") == 9728:
            filt = RT_FILTER_NEAREST
        src = tex["source"]
        if src not in decoded:
            v = doc["bufferViews"][doc["images"][src]["bufferView"]]
            off = v.get("byteOffset", 0)
            decoded[src] = png_decode_rgba8(binary[off:off + v["byteLength"]])
        images.append((decoded[src], fmt, filt))
        return len(images) - 1

    def colour(rgba):
        images.append((np.array(rgba, np.float32).reshape(1, 1, 4), RT_FORMAT_R32G32B32A32_SFLOAT, RT_FILTER_NEAREST))
        return len(images) - 1

    for mat in doc.get("materials", []):
        pbr = mat.get("pbrMetallicRoughness", {})
        g = {"indices": [], "opaque": mat.get("alphaMode", "OPAQUE") == "OPAQUE"}
        g["diffuse"] = texture(pbr["baseColorTexture"], RT_FORMAT_R8G8B8A8_SRGB) if "baseColorTexture" in pbr \
            else colour(pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0]))
        g["metallic_roughness"] = texture(pbr["metallicRoughnessTexture"], RT_FORMAT_R8G8B8A8_SRGB) \
            if "metallicRoughnessTexture" in pbr \
            else colour([1.0, pbr.get("roughnessFactor", 1.0), pbr.get("metallicFactor", 1.0), 1.0])
        g["normal_map"] = texture(mat["normalTexture"], RT_FORMAT_R8G8B8A8_UNORM) if "normalTexture" in mat else -1
        geoms.append(g)
    if not geoms:
        geoms.append({"indices": [], "opaque": True, "diffuse": -1, "metallic_roughness": colour([1.0, 1.0, 0.0, 1.0]),
                      "normal_map": -1})
    pos, nrm, uv = [], [], []
    base = 0
    for mesh in doc.get("meshes", []):
        for prim in mesh["primitives"]:
            g = geoms[prim.get("material", 0)]
            idx = _accessor(doc, binary, prim["indices"]).reshape(-1).astype(np.uint32) + np.uint32(base)
            g["indices"].append(idx)
            p = _accessor(doc, binary, prim["attributes"]["POSITION"]).astype(np.float32)
            n = _accessor(doc, binary, prim["attributes"]["NORMAL"]).astype(np.float32)
            t_acc = doc["accessors"][prim["attributes"]["TEXCOORD_0"]]
            t = _accessor(doc, binary, prim["attributes"]["TEXCOORD_0"])
            if t_acc["componentType"] == 5121:
                t = t.astype(np.float32) / np.float32(255.0)
            elif t_acc["componentType"] == 5123:
                t = t.astype(np.float32) / np.float32(65535.0)
            pos.append(p), nrm.append(n), uv.append(t.astype(np.float32))
            base += len(p)
    for g in geoms:
        g["indices"] = (np.concatenate(g["indices"]) if g["indices"] else np.zeros(0, np.uint32)).reshape(-1, 3)
    cat = (lambda xs, k: np.concatenate(xs) if xs else np.zeros((0, k), np.float32))
    return {"positions": cat(pos, 3), "normals": cat(nrm, 3), "uvs": cat(uv, 2), "geometries": geoms,
            "images": images}
