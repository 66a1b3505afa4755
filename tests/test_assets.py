"""Asset decoding (include/rtassets.h): PNG -> RGBA8 and GLB -> model arrays.

Host code of librtcore.so, so these run on the CPU.  Three checks: the
native decoders against the committed fixtures (whose expected arrays are the
encoded samples themselves), the oracle against the same fixtures, and the
native decoders against the oracle on the reference's own asset files when
RT_REFERENCE_RESOURCES names a checkout's resources/ folder.  Malformed files
must fail with a status, never crash.
"""
import ctypes as C
import os
from pathlib import Path

import numpy as np
import pytest

from oracle import assets_oracle as AO
from rtgallery import abi, assets

FIX = Path(__file__).resolve().parent / "golden" / "asset_fixtures.npz"
# The reference's own resources/ folder, when a checkout of it is available:
# set RT_REFERENCE_RESOURCES to that folder to run the tests that decode its
# PNG and GLB files; they are skipped otherwise.
_REF_ENV = os.environ.get("RT_REFERENCE_RESOURCES", "")
REF_RESOURCES = Path(_REF_ENV) if _REF_ENV else None


@pytest.fixture(scope="module")
def fixtures(rtlib):
    return np.load(FIX)


def _png_names(fx):
    return sorted(k.split("/", 1)[1] for k in fx.files if k.startswith("png/"))


def test_png_fixtures_native(fixtures):
    names = _png_names(fixtures)
    assert len(names) >= 35
    for n in names:
        got = assets.decode_png(fixtures[f"png/{n}"].tobytes())
        exp = fixtures[f"png_rgba/{n}"]
        assert got.shape == exp.shape, n
        assert (got == exp).all(), f"{n}: {int((got != exp).any(-1).sum())} texels differ"


def test_png_fixtures_oracle(fixtures):
    for n in _png_names(fixtures):
        assert (AO.png_decode_rgba8(fixtures[f"png/{n}"].tobytes()) == fixtures[f"png_rgba/{n}"]).all(), n


def test_png_header_query(fixtures, rtlib):
    data = fixtures["png/c6_d16_adam7"].tobytes()
    w, h = C.c_uint32(), C.c_uint32()
    assert rtlib.rt_png_decode_rgba8(data, len(data), None, 0, C.byref(w), C.byref(h)) == abi.RT_OK
    assert (w.value, h.value) == (13, 11)
    small = np.empty(13 * 11 * 4 - 1, np.uint8)
    assert rtlib.rt_png_decode_rgba8(data, len(data), small.ctypes.data, small.nbytes, C.byref(w),
                                     C.byref(h)) == abi.RT_ERR_INVALID
    assert b"needed" in rtlib.rt_last_error_string()


def _decode_status(rtlib, data: bytes) -> int:
    w, h = C.c_uint32(), C.c_uint32()
    out = np.empty(1 << 20, np.uint8)
    return rtlib.rt_png_decode_rgba8(data, len(data), out.ctypes.data, out.nbytes, C.byref(w), C.byref(h))


def test_png_malformed_inputs_fail_cleanly(fixtures, rtlib):
    good = fixtures["png/c2_d8_plain"].tobytes()
    assert _decode_status(rtlib, good) == abi.RT_OK
    cases = {
        "empty": b"",
        "signature": b"\x88" + good[1:],
        "truncated": good[:-20],
        "crc": good[:40] + bytes([good[40] ^ 0x55]) + good[41:],
        "no_iend": good[:-12],
    }
    for name, data in cases.items():
        st = _decode_status(rtlib, data)
        assert st in (abi.RT_ERR_INVALID, abi.RT_ERR_UNSUPPORTED), (name, st)
    # a bad filter byte / adler / deflate stream behind valid CRCs
    from rtgallery.assets import encode_png

    s = np.arange(4 * 5 * 3, dtype=np.uint8).reshape(4, 5, 3)
    bad_filter = encode_png(s, 2, filters=(7,))
    assert _decode_status(rtlib, bad_filter) == abi.RT_ERR_INVALID
    assert b"filter" in rtlib.rt_last_error_string()
    pal = np.zeros((2, 3), np.uint8)
    bad_index = encode_png(np.full((2, 2, 1), 3), 3, 2, palette=pal)
    assert _decode_status(rtlib, bad_index) == abi.RT_ERR_INVALID


def test_png_random_corruption_never_crashes(fixtures, rtlib):
    """Byte flips inside the compressed data (CRCs recomputed, so the
    decoder reaches the inflater and the unfilter) give a status or the
    right size, never a crash."""
    import struct
    import zlib

    rng = np.random.default_rng(7)
    src = fixtures["png/c6_d8_adam7"].tobytes()
    at = 8
    chunks = []
    while at < len(src):
        (n,) = struct.unpack_from(">I", src, at)
        chunks.append((src[at + 4:at + 8], bytearray(src[at + 8:at + 8 + n])))
        at += 12 + n
    statuses = set()
    for _ in range(300):
        out = b"\x89PNG\r\n\x1a\n"
        for kind, body in chunks:
            b = bytearray(body)
            if kind == b"IDAT":
                for _k in range(int(rng.integers(1, 4))):
                    b[int(rng.integers(0, len(b)))] ^= int(rng.integers(1, 256))
            out += struct.pack(">I", len(b)) + kind + bytes(b) + struct.pack(">I", zlib.crc32(kind + b) & 0xFFFFFFFF)
        statuses.add(_decode_status(rtlib, out))
    assert statuses <= {abi.RT_OK, abi.RT_ERR_INVALID, abi.RT_ERR_UNSUPPORTED}
    assert abi.RT_ERR_INVALID in statuses


def _glb_names(fx):
    return sorted(k.split("/", 1)[1] for k in fx.files if k.startswith("glb/"))


def _check_glb(d: dict, fixtures, name: str):
    e = lambda k: fixtures[f"glb_exp/{name}/{k}"]  # noqa: E731
    assert (d["positions"] == e("positions")).all() and (d["normals"] == e("normals")).all()
    assert (d["uvs"] == e("uvs")).all()
    slots = e("slots")
    assert len(d["geometries"]) == len(slots)
    for gi, g in enumerate(d["geometries"]):
        assert (np.asarray(g["indices"]).reshape(-1) == e(f"indices{gi}").reshape(-1)).all(), (name, gi)
        assert bool(g["opaque"]) == bool(e("opaque")[gi])
        assert [g["diffuse"], g["metallic_roughness"], g["normal_map"]] == list(slots[gi])
    assert len(d["images"]) == len(e("formats"))
    for k, im in enumerate(d["images"]):
        tex, fmt, filt = (im.texels, im.format, im.filter) if hasattr(im, "texels") else im
        assert fmt == e("formats")[k] and filt == e("filters")[k], (name, k)
        assert (np.asarray(tex).reshape(e(f"image{k}").shape) == e(f"image{k}")).all(), (name, k)


def test_glb_fixtures_native_and_oracle(fixtures):
    names = _glb_names(fixtures)
    assert len(names) == 2
    for n in names:
        data = fixtures[f"glb/{n}"].tobytes()
        _check_glb(assets.read_glb(data), fixtures, n)
        _check_glb(AO.glb_decode(data), fixtures, n)


def test_glb_load_pushes_images_in_reference_order(fixtures):
    tex = assets.TextureTable()
    tex.push_image(assets.Texture(np.zeros((1, 1, 4), np.uint8), abi.RT_FORMAT_R8G8B8A8_SRGB))
    m = assets.load_glb(fixtures["glb/two_materials"].tobytes(), "m", 0, tex)
    assert len(tex) == 6
    g0, g1 = m.geometries
    assert (g0.diffuse_image, g0.metallic_roughness_image, g0.normal_map_image) == (1, 2, -1)
    assert (g1.diffuse_image, g1.metallic_roughness_image, g1.normal_map_image) == (3, 4, 5)
    assert not g0.opaque and g1.opaque
    m2 = assets.load_glb(fixtures["glb/interleaved_no_material"].tobytes(), "n", 0, tex)
    assert m2.geometries[0].diffuse_image == 0 and m2.geometries[0].metallic_roughness_image == 6


def test_glb_malformed_inputs_fail_cleanly(fixtures, rtlib):
    import json
    import struct

    good = fixtures["glb/two_materials"].tobytes()
    h = C.c_void_p()

    def status(data):
        st = rtlib.rt_glb_load(data, len(data), C.byref(h))
        if st == abi.RT_OK:
            rtlib.rt_glb_destroy(h)
        return st

    assert status(good) == abi.RT_OK
    assert status(b"") == abi.RT_ERR_INVALID
    assert status(good[:30]) == abi.RT_ERR_INVALID
    jl = struct.unpack_from("<I", good, 12)[0]
    doc = json.loads(good[20:20 + jl])
    binary = good[20 + jl + 8:]

    def with_doc(mut):
        d = json.loads(json.dumps(doc))
        mut(d)
        from rtgallery.assets import encode_glb

        return encode_glb(d, binary)

    def uri_image(d):
        d["images"][0] = {"uri": "x.png"}

    def out_of_range(d):
        d["accessors"][0]["count"] = 10 ** 6

    def missing_normal(d):
        del d["meshes"][0]["primitives"][0]["attributes"]["NORMAL"]

    def lines(d):
        d["meshes"][0]["primitives"][0]["mode"] = 1

    def bad_index(d):
        d["meshes"][1]["primitives"][0]["material"] = 9

    expect = {uri_image: abi.RT_ERR_UNSUPPORTED, out_of_range: abi.RT_ERR_INVALID,
              missing_normal: abi.RT_ERR_INVALID, lines: abi.RT_ERR_UNSUPPORTED, bad_index: abi.RT_ERR_INVALID}
    for mut, code in expect.items():
        assert status(with_doc(mut)) == code, mut.__name__
    rng = np.random.default_rng(3)
    for _ in range(200):
        b = bytearray(good)
        for _k in range(int(rng.integers(1, 6))):
            b[int(rng.integers(0, len(b)))] ^= int(rng.integers(1, 256))
        assert status(bytes(b)) in (abi.RT_OK, abi.RT_ERR_INVALID, abi.RT_ERR_UNSUPPORTED, abi.RT_ERR_TOO_LARGE)


def test_standin_default_scene_assets():
    a = assets.standin_assets()
    assert set(a) == set(assets.DEFAULT_ASSETS)
    sc = assets.default_scene(a, 64, 36)
    assert [m.triangle_count for m in sc.models] == [2, 2304, 45448, 2]
    assert len(sc.instances) == 105 and len(sc.textures) == 10
    assert sc.textures[3].filter == abi.RT_FILTER_LINEAR and sc.textures[2].format == abi.RT_FORMAT_R8G8B8A8_UNORM
    fence = sc.models[3].geometries[0]
    assert not fence.opaque and sc.textures[fence.diffuse_image].texels.shape == (256, 256, 4)
    # plane and tori have no materials: fallback diffuse images 0 and 1
    assert sc.models[0].geometries[0].diffuse_image == 0 and sc.models[1].geometries[0].diffuse_image == 1
    for name in ("plane.glb", "tori.glb", "lain.glb", "fence.glb"):
        n, o = assets.read_glb(a[name]), AO.glb_decode(a[name])
        assert (n["positions"] == o["positions"]).all() and (n["uvs"] == o["uvs"]).all()
        assert all((g["indices"] == h["indices"]).all() for g, h in zip(n["geometries"], o["geometries"]))
    # the figure turns by 0.05 rad per frame; nothing else moves
    i0, i5 = assets.default_scene_instances(0, 0), assets.default_scene_instances(0, 5)
    moved = (i0["transform"] != i5["transform"]).any(axis=(1, 2))
    assert list(np.nonzero(moved)[0]) == [2]


needs_reference = pytest.mark.skipif(REF_RESOURCES is None or not (REF_RESOURCES / "lain.glb").exists(),
                                     reason="RT_REFERENCE_RESOURCES does not name the reference's resources/")


@needs_reference
@pytest.mark.parametrize("name", ["blue_noise_64x64.png", "green.png", "pink.png", "flipped_ggx_lut.png"])
def test_reference_png_native_equals_oracle(name):
    data = (REF_RESOURCES / name).read_bytes()
    assert (assets.decode_png(data) == AO.png_decode_rgba8(data)).all()


@needs_reference
@pytest.mark.parametrize("name,tris,opaque,images",
                         [("plane.glb", 2, [True], 1), ("tori.glb", 2304, [True], 1),
                          ("lain.glb", 45448, [True], 2), ("fence.glb", 2, [False], 2)])
def test_reference_glb_native_equals_oracle(name, tris, opaque, images):
    data = (REF_RESOURCES / name).read_bytes()
    n = assets.read_glb(data)
    assert n["triangle_count"] == tris
    assert [g["opaque"] for g in n["geometries"]] == opaque and len(n["images"]) == images
    if name == "lain.glb":    # the 2048x2048 texture would take the pure-Python oracle minutes
        assert n["images"][0].texels.shape == (2048, 2048, 4) and n["images"][0].filter == abi.RT_FILTER_LINEAR
        return
    o = AO.glb_decode(data)
    assert (n["positions"] == o["positions"]).all() and (n["normals"] == o["normals"]).all()
    assert (n["uvs"] == o["uvs"]).all()
    for g, h in zip(n["geometries"], o["geometries"]):
        assert (g["indices"] == h["indices"]).all()
    for im, (tex, fmt, filt) in zip(n["images"], o["images"]):
        assert im.format == fmt and im.filter == filt and (im.texels == tex).all()
