"""CPU tests of the oracle: the reference's own known-answer test, published
vectors, and properties the oracle must have before it can check the GPU."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import abi, scenes

GOLDEN = Path(__file__).resolve().parent / "golden"


# ---------------------------------------------------------------------------
# the reference's unit test (shaders/ray-tracing/src/pbr.rs:52-69)
# ---------------------------------------------------------------------------
def _dot(a, b):
    return float(np.float32(np.float32(a[0] * b[0]) + np.float32(a[1] * b[1])) + np.float32(a[2] * b[2]))


@pytest.mark.parametrize("eps_key", ["nov_epsilon_rust", "nov_epsilon_glsl"])
@pytest.mark.parametrize("dbl", [False, True])
def test_ggx_division_by_zero_kat(eps_key, dbl):
    kat = json.loads((GOLDEN / "ggx_division_by_zero.json").read_text())
    n, v, l = kat["normal"], kat["view"], kat["light"]
    nov = min(max(_dot(n, v), kat[eps_key]), 1.0)
    nol = min(max(_dot(n, l), 0.0), 1.0)
    out = O.debug_eval(abi.RT_FN_V_SMITH_GGX_CORRELATED, np.array([nov, nol, kat["roughness"]]), 1, 1, dbl)
    assert math.isfinite(out[0]), out
    # the closed form at these inputs: 0.5 / (NoL*NoV + NoV*NoL)
    assert out[0] == pytest.approx(0.5 / (2 * np.float32(nov)), rel=1e-6)


def test_brdf_at_ggx_kat_inputs_is_finite():
    # full brdf (pbr.glsl:174-211) with the KAT's vectors; the GLSL clamp 1e-9
    p = np.zeros(16, np.float32)
    p[0:3] = [0, 1, 0]
    p[3:6] = [1, 0, 0]
    p[6:9] = [0, 1, 0]
    p[9] = 0.3  # roughness 0 makes D_GGX 0/0 in the reference; 0.3 keeps it defined
    p[10:13] = [0.5, 0.5, 0.5]
    p[13], p[14] = 0.0, 1.0
    for dbl in (False, True):
        out = O.debug_eval(abi.RT_FN_BRDF, p, 1, 3, dbl)
        assert np.isfinite(out).all()


# ---------------------------------------------------------------------------
# published vectors
# ---------------------------------------------------------------------------
def test_pcg32_published_vector():
    kat = json.loads((GOLDEN / "pcg32_kat.json").read_text())
    r = scenes.Pcg32(kat["seed"], kat["seq"])
    assert [r.next_u32() for _ in kat["outputs"]] == kat["outputs"]


def test_pcg32_vectorised_matches_scalar():
    a = scenes.Pcg32(7, 3)
    b = scenes.Pcg32(7, 3)
    v = a.u32_array(70000)
    s = np.array([b.next_u32() for _ in range(70000)], np.uint32)
    assert (v == s).all() and a.state == b.state


def test_srgb_transfer_known_values():
    x = np.array([0.0, 0.0031308, 0.5, 1.0, 0.001], np.float32)
    out = O.debug_eval(abi.RT_FN_LINEAR_TO_SRGB, x, len(x), 1)
    assert out[0] == 0.0
    assert out[1] == pytest.approx(0.0031308 * 12.92, rel=1e-6)
    assert out[2] == pytest.approx(0.735356983, abs=2e-6)   # IEC 61966-2-1 at 0.5
    assert out[3] == pytest.approx(1.0, abs=1e-6)
    assert out[4] == pytest.approx(0.01292, rel=1e-5)


def test_heatmap_palette_endpoints():
    out = O.debug_eval(abi.RT_FN_HEATMAP, np.array([0.0, 0.05, 0.5, 1.0], np.float32), 4, 3).reshape(4, 3)
    assert np.all((out >= 0) & (out <= 1))
    # at heat 0 the palette blends colours[0] (and its blurred neighbours)
    assert out[0][2] > out[0][0]
    # at heat 1 the last stop dominates (red-magenta)
    assert out[3][0] > out[3][1]


# ---------------------------------------------------------------------------
# the oracle's own arithmetic
# ---------------------------------------------------------------------------
def test_sincos_accuracy():
    x = np.linspace(-50, 50, 20001).astype(np.float32)
    out = O.debug_eval(abi.RT_FN_SINCOS, x, len(x), 2).reshape(-1, 2)
    ref = np.stack([np.sin(x.astype(np.float64)), np.cos(x.astype(np.float64))], 1)
    assert np.abs(out - ref).max() < 4e-7


def test_world_to_object_inverse():
    rng = scenes.Pcg32(3)
    for _ in range(50):
        m = scenes.affine(scenes.random_rotation(rng), [rng.uniform_range(-9, 9) for _ in range(3)],
                          rng.uniform_range(0.1, 5.0))
        w, ok = O.world_to_object(m)
        assert ok
        full = np.vstack([m, [0, 0, 0, 1]])
        inv = np.linalg.inv(full)[:3]
        assert np.allclose(w.reshape(3, 4), inv, atol=1e-5 * max(1, np.abs(inv).max()))
    w, ok = O.world_to_object(np.zeros((3, 4)))
    assert not ok


def _wt(o, d, tri, tmin=0.0):
    p = np.zeros(16, np.float32)
    p[0:3], p[3:6] = o, d
    p[6:15] = np.asarray(tri, np.float32).reshape(9)
    p[15] = tmin
    return O.debug_eval(abi.RT_FN_WATERTIGHT, p, 1, 4)


def test_watertight_known_hit():
    out = _wt([0.2, 0.2, 1.0], [0, 0, -1], [[0, 0, 0], [1, 0, 0], [0, 1, 0]])
    assert out[0] != 0 and out[1] == pytest.approx(1.0) and out[2] == pytest.approx(0.2) and out[3] == pytest.approx(0.2)
    assert _wt([2.0, 2.0, 1.0], [0, 0, -1], [[0, 0, 0], [1, 0, 0], [0, 1, 0]])[0] == 0


def test_watertight_shared_edges_never_leak():
    """Rays aimed at the shared diagonal of a flat quad hit at least one of
    its two triangles (the union is flat around the diagonal, so exact
    geometry hits; the test must not leak through the edge)."""
    rng = np.random.default_rng(0)
    a, b, c, d = np.array([[0, 0, 0], [1, 0.1, 0], [1.2, 1, 0], [0.1, 0.9, 0]], np.float32)
    t1, t2 = [a, b, c], [a, c, d]
    leaks = both = 0
    for _ in range(400):
        s = np.float32(0.02 + 0.96 * rng.random())
        p = (a + s * (c - a)).astype(np.float32)
        o = (p + rng.normal(size=3) * 3).astype(np.float32)
        dvec = (p - o).astype(np.float32)
        h1 = _wt(o, dvec, t1)[0] != 0
        h2 = _wt(o, dvec, t2)[0] != 0
        leaks += not (h1 or h2)
        both += h1 and h2
    assert leaks == 0


def test_watertight_fan_vertex_never_leaks():
    """Rays through the centre vertex of a closed fan hit some triangle."""
    rng = np.random.default_rng(1)
    k = 7
    ang = np.sort(rng.random(k)) * 2 * np.pi
    rim = np.stack([np.cos(ang), np.sin(ang), np.zeros(k)], 1).astype(np.float32)
    centre = np.zeros(3, np.float32)
    tris = [[centre, rim[i], rim[(i + 1) % k]] for i in range(k)]
    for _ in range(300):
        o = (rng.normal(size=3) * 4).astype(np.float32)
        if abs(o[2]) < 0.1:
            continue
        dvec = (centre - o).astype(np.float32)
        assert any(_wt(o, dvec, t)[0] != 0 for t in tris)


def _random_rays(n, seed, box, lo=0.0, hi=1e4):
    r = scenes.random_rays(n, seed, box)
    r["tmin"], r["tmax"] = lo, hi
    return r


@pytest.mark.parametrize("scene_fn", [lambda: scenes.scene_small(64, 64), lambda: scenes.scene_gallery(64, 48)])
def test_oracle_bvh_matches_bruteforce(scene_fn):
    sc = scene_fn()
    bvh = O.OracleScene(sc)
    brute = O.OracleScene(sc, bruteforce=True)
    rays = _random_rays(3000, 11, 16.0)
    for flags in (0, abi.RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT | abi.RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER):
        h1, _ = bvh.trace(rays, ray_flags=flags)
        h2, _ = brute.trace(rays, ray_flags=flags)
        if flags:
            assert ((h1["instance_id"] == 0xFFFFFFFF) == (h2["instance_id"] == 0xFFFFFFFF)).all()
        else:
            assert (h1.view(np.uint32) == h2.view(np.uint32)).all()
    # the rendered image through either structure is identical too
    i1, r1, s1 = bvh.render(width=48, height=32)
    i2, r2, s2 = brute.render(width=48, height=32)
    assert (i1 == i2).all() and (r1 == r2).all() and s1["traversals"] == s2["traversals"]


def test_golden_small_rays_oracle():
    g = np.load(GOLDEN / "small_rays.npz")
    sc = _scene_from_golden(g)
    hits, _ = O.OracleScene(sc).trace(g["rays"])
    assert (hits.view(np.uint32) == g["hits"].view(np.uint32)).all()
    assert (hits["instance_id"] != 0xFFFFFFFF).sum() > 500


def _scene_from_golden(g):
    tor = scenes.Model(g["torus_positions"], g["torus_normals"], g["torus_uvs"],
                       [scenes.Geometry(g["torus_indices"], True, scenes.TEX_DIFFUSE_A, scenes.TEX_MR_DEFAULT)])
    gnd = scenes.Model(g["ground_positions"], g["ground_normals"], g["ground_uvs"],
                       [scenes.Geometry(g["ground_indices"], True, scenes.TEX_DIFFUSE_B, scenes.TEX_MR_DEFAULT)])
    base = scenes.scene_small(64, 32)
    return scenes.Scene([tor, gnd], base.textures, g["instances"], base.uniforms, 64, 32, 3, 1)


def test_fp64_shading_close_to_fp32():
    sc = scenes.scene_gallery(64, 40)
    o = O.OracleScene(sc)
    _, r32, s32 = o.render()
    _, r64, s64 = o.render(double=True)
    assert s32["traversals"] == s64["traversals"]
    assert np.abs(r32 - r64).max() < 1e-4


def test_alpha_clip_changes_hits():
    """The fence's checker alpha removes candidates (any_hit_alpha_clip.glsl)."""
    sc = scenes.scene_gallery(32, 32)
    o = O.OracleScene(sc)
    ys, xs = np.mgrid[0:40, 0:40]
    rays = np.zeros(1600, abi.RAY_DTYPE)
    rays["origin"] = np.stack([2 - 1 + xs.ravel() * 0.05, 0.05 + ys.ravel() * 0.023, np.full(1600, 0.0)], 1)
    rays["direction"] = [0, 0, 1]
    rays["tmin"], rays["tmax"] = 0.0, 100.0
    with_ah, _ = o.trace(rays)
    opaque, _ = o.trace(rays, ray_flags=abi.RT_RAY_FLAG_OPAQUE)
    fence = 3
    n_ah = (with_ah["instance_id"] == fence).sum()
    n_op = (opaque["instance_id"] == fence).sum()
    assert n_op > 0 and 0.25 * n_op < n_ah < 0.75 * n_op
