"""Generates tests/golden/asset_fixtures.npz: PNG and GLB files with the
arrays they must decode to.

Every fixture is written from known samples by the package's own writers
(rtgallery.assets.encode_png / GlbBuilder, or a hand-laid GLB below), so the
expected output is the input itself, expanded to RGBA8 by the PNG rules
(grey g -> g,g,g,255; RGB -> alpha 255; palette through PLTE / tRNS; tRNS
colour keys -> alpha 0; samples below 8 bits scaled to 0..255; 16-bit
samples keep their high byte).  No decoder is involved in making them.

PNG cases: every colour type x bit depth of the PNG specification, plain and
Adam7-interlaced, odd sizes (13x11, partial Adam7 passes), all five row
filters, grey / RGB / palette transparency, several IDAT chunks, stored and
fixed-Huffman deflate blocks, ancillary chunks.
GLB cases: two materials (texture with a LINEAR sampler; colour factor,
NEAREST metallic-roughness texture and a normal map), a primitive without a
material, u8 / u16 / u32 indices, interleaved vertex data (byteStride),
normalized u16 texture coordinates, a file without materials.

Regenerate with ``python tests/golden/make_asset_fixtures.py``.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def _expand(samples: np.ndarray, color: int, depth: int, palette=None, trns=None) -> np.ndarray:
    s = samples.astype(np.int64)
    if s.ndim == 2:
        s = s[:, :, None]
    h, w, _ = s.shape
    if depth == 16:
        to8 = s >> 8
    elif depth == 8:
        to8 = s
    else:
        to8 = s * (255 // ((1 << depth) - 1))
    out = np.zeros((h, w, 4), np.int64)
    if color == 0:
        out[..., 0] = out[..., 1] = out[..., 2] = to8[..., 0]
        out[..., 3] = 255
        if trns is not None:
            out[..., 3] = np.where(s[..., 0] == (trns[0] << 8 | trns[1]), 0, 255)
    elif color == 2:
        out[..., :3] = to8
        out[..., 3] = 255
        if trns is not None:
            key = [trns[k] << 8 | trns[k + 1] for k in (0, 2, 4)]
            out[..., 3] = np.where((s == np.array(key)).all(-1), 0, 255)
    elif color == 3:
        pal = np.asarray(palette, np.int64).reshape(-1, 3)
        out[..., :3] = pal[s[..., 0]]
        alpha = np.full(len(pal), 255)
        if trns is not None:
            alpha[:len(trns)] = list(trns)
        out[..., 3] = alpha[s[..., 0]]
    elif color == 4:
        out[..., 0] = out[..., 1] = out[..., 2] = to8[..., 0]
        out[..., 3] = to8[..., 1]
    else:
        out[...] = to8
    return out.astype(np.uint8)


def png_cases(rng) -> dict:
    from rtgallery.assets import encode_png

    cases = {}
    combos = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
              (4, 8), (4, 16), (6, 8), (6, 16)]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
    for color, depth in combos:
        for interlace in (False, True):
            h, w = 11, 13
            hi = (1 << depth) - 1
            if color == 3:
                npal = min(1 << depth, 7 if depth > 2 else (1 << depth))
                s = rng.integers(0, npal, (h, w, 1))
                pal = rng.integers(0, 256, (npal, 3))
                trns = bytes(rng.integers(0, 256, max(1, npal - 2)).astype(np.uint8))
                data = encode_png(s, color, depth, interlace, palette=pal, trns=trns)
                exp = _expand(s, color, depth, pal, trns)
            else:
                s = rng.integers(0, hi + 1, (h, w, ch[color]))
                data = encode_png(s, color, depth, interlace)
                exp = _expand(s, color, depth)
            name = f"c{color}_d{depth}_{'adam7' if interlace else 'plain'}"
            cases[name] = (data, exp)
    # colour-key transparency (grey 8 / 16, RGB 8 / 16)
    for color, depth in ((0, 8), (0, 16), (0, 2), (2, 8), (2, 16)):
        hi = (1 << depth) - 1
        s = rng.integers(0, min(hi, 5) + 1, (9, 10, ch[color]))
        key = s[0, 0]
        trns = b"".join(int(k).to_bytes(2, "big") for k in key)
        cases[f"trns_c{color}_d{depth}"] = (encode_png(s, color, depth, trns=trns),
                                            _expand(s, color, depth, trns=trns))
    # deflate block kinds and chunking
    s = rng.integers(0, 256, (20, 17, 4))
    cases["stored_blocks"] = (encode_png(s, 6, level=0), _expand(s, 6, 8))
    s = rng.integers(0, 4, (8, 8, 3)) * 60          # short repetitive data: fixed-Huffman blocks
    cases["fixed_huffman"] = (encode_png(s, 2, level=9, filters=(0,)), _expand(s, 2, 8))
    s = rng.integers(0, 65536, (24, 31, 4))
    cases["multi_idat_adam7_rgba16"] = (encode_png(s, 6, 16, True, idat_split=97,
                                                   extra_chunks=((b"tEXt", b"Comment\0fixture"),
                                                                 (b"pHYs", bytes(9)))), _expand(s, 6, 16))
    s = rng.integers(0, 2, (5, 301, 1))
    cases["wide_1bit_each_filter"] = (encode_png(s, 0, 1, filters=(4, 3, 2, 1, 0)), _expand(s, 0, 1))
    return cases


def glb_cases(rng) -> dict:
    """name -> (bytes, expected dict)."""
    from rtgallery.assets import GlbBuilder, encode_glb, encode_png

    out = {}
    # 1) two materials, three primitives (u16, u32, u8 indices), one without material
    b = GlbBuilder()
    t0 = rng.integers(0, 256, (6, 5, 4))
    t1 = rng.integers(0, 256, (4, 4, 3))
    t2 = rng.integers(0, 256, (3, 7, 4))
    tex0 = b.image(encode_png(t0, 6), 9729)
    tex1 = b.image(encode_png(t1, 2), 9728)
    tex2 = b.image(encode_png(t2, 6), None)
    m0 = b.material(pbrMetallicRoughness={"baseColorTexture": {"index": tex0}, "metallicFactor": 0.25,
                                          "roughnessFactor": 0.75}, alphaMode="MASK", alphaCutoff=0.5)
    m1 = b.material(pbrMetallicRoughness={"baseColorFactor": [0.1, 0.2, 0.3, 0.4],
                                          "metallicRoughnessTexture": {"index": tex1}},
                    normalTexture={"index": tex2}, alphaMode="OPAQUE")
    verts, idxs, geos = [], [], {0: [], 1: []}
    base = 0
    for k, (mat, itype, nv, nt) in enumerate([(m1, 5123, 9, 7), (m0, 5125, 6, 4), (None, 5121, 5, 3)]):
        p = rng.standard_normal((nv, 3)).astype(np.float32)
        n = rng.standard_normal((nv, 3)).astype(np.float32)
        t = rng.random((nv, 2)).astype(np.float32)
        i = rng.integers(0, nv, (nt, 3))
        b.mesh(p, n, t, i, material=mat, index_type=itype, node={"translation": [k, 2 * k, 0]})
        verts.append((p, n, t))
        geos[0 if mat in (None, m0) else 1].append(i + base)
        base += nv
    exp = {"positions": np.concatenate([v[0] for v in verts]), "normals": np.concatenate([v[1] for v in verts]),
           "uvs": np.concatenate([v[2] for v in verts]),
           "indices0": np.concatenate(geos[0]).astype(np.uint32), "indices1": np.concatenate(geos[1]).astype(np.uint32),
           "opaque": np.array([0, 1]), "slots": np.array([[0, 1, -1], [2, 3, 4]]),
           "formats": np.array([43, 109, 109, 43, 37]), "filters": np.array([1, 0, 0, 0, 1]),
           "image0": _expand(t0, 6, 8), "image1": np.array([1.0, 0.75, 0.25, 1.0], np.float32),
           "image2": np.array([0.1, 0.2, 0.3, 0.4], np.float32), "image3": _expand(t1, 2, 8),
           "image4": _expand(t2, 6, 8)}
    out["two_materials"] = (b.encode(), exp)

    # 2) interleaved vertices (byteStride 32), normalized u16 uvs, no materials
    nv, nt = 11, 9
    p = rng.standard_normal((nv, 3)).astype(np.float32)
    n = rng.standard_normal((nv, 3)).astype(np.float32)
    uvq = rng.integers(0, 65536, (nv, 2)).astype(np.uint16)
    inter = np.zeros((nv, 32), np.uint8)
    inter[:, 0:12] = p.view(np.uint8).reshape(nv, 12)
    inter[:, 12:24] = n.view(np.uint8).reshape(nv, 12)
    inter[:, 24:28] = uvq.view(np.uint8).reshape(nv, 4)
    idx = rng.integers(0, nv, (nt, 3)).astype(np.uint16)
    binary = inter.tobytes() + idx.tobytes()
    doc = {"asset": {"version": "2.0"}, "buffers": [{"byteLength": len(binary)}],
           "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": inter.nbytes, "byteStride": 32},
                           {"buffer": 0, "byteOffset": inter.nbytes, "byteLength": idx.nbytes}],
           "accessors": [{"bufferView": 0, "byteOffset": 0, "componentType": 5126, "count": nv, "type": "VEC3"},
                         {"bufferView": 0, "byteOffset": 12, "componentType": 5126, "count": nv, "type": "VEC3"},
                         {"bufferView": 0, "byteOffset": 24, "componentType": 5123, "count": nv, "type": "VEC2",
                          "normalized": True},
                         {"bufferView": 1, "componentType": 5123, "count": nt * 3, "type": "SCALAR"}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2},
                                       "indices": 3, "mode": 4}]}]}
    exp = {"positions": p, "normals": n, "uvs": uvq.astype(np.float32) / np.float32(65535.0),
           "indices0": idx.astype(np.uint32), "opaque": np.array([1]), "slots": np.array([[-1, 0, -1]]),
           "formats": np.array([109]), "filters": np.array([0]), "image0": np.array([1.0, 1.0, 0.0, 1.0], np.float32)}
    out["interleaved_no_material"] = (encode_glb(doc, binary), exp)
    return out


def main() -> None:
    rng = np.random.default_rng(20261204)
    arrays = {}
    for name, (data, exp) in png_cases(rng).items():
        arrays[f"png/{name}"] = np.frombuffer(data, np.uint8)
        arrays[f"png_rgba/{name}"] = exp
    for name, (data, exp) in glb_cases(rng).items():
        arrays[f"glb/{name}"] = np.frombuffer(data, np.uint8)
        for k, v in exp.items():
            arrays[f"glb_exp/{name}/{k}"] = v
    np.savez_compressed(HERE / "asset_fixtures.npz", **arrays)
    print(json.dumps({"files": len([k for k in arrays if k.startswith(("png/", "glb/"))]),
                      "bytes": (HERE / "asset_fixtures.npz").stat().st_size}))


if __name__ == "__main__":
    import __graft_entry__

    __graft_entry__.load_package()
    main()
