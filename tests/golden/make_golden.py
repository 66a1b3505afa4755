"""Generates the committed golden fixtures in this directory.

* ggx_division_by_zero.json — the reference's only unit test
  (shaders/ray-tracing/src/pbr.rs:52-69): V_SmithGGXCorrelated with
  view (1,0,0), light (0,1,0), normal (0,1,0), roughness 0 must be finite.
  The inputs are copied from that test; both NoV epsilons are recorded
  (1e-10 in pbr.rs:24-35, 1e-9 = 10.0e-10 in shaders/pbr.glsl:33).
* pcg32_kat.json — the published first outputs of PCG32 seeded (42, 54)
  (O'Neill's pcg32 demo), pinning the scene generator's RNG.
* small_rays.npz — a small self-contained case: a 64x32 torus and a ground
  quad instanced as in the small benchmark scene, 2048 rays (camera rays and
  random rays, some from inside objects), and the oracle's hits.  Storing
  the inputs makes GPU tests independent of the platform's libm (the scene
  generator uses numpy sin/cos).  Regenerate with
  ``python tests/golden/make_golden.py`` (needs the oracle, gcc).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def ggx_kat() -> dict:
    return {
        "source": "shaders/ray-tracing/src/pbr.rs:52-69 (test_ggx_division_by_zero)",
        "view": [1.0, 0.0, 0.0],
        "light": [0.0, 1.0, 0.0],
        "normal": [0.0, 1.0, 0.0],
        "roughness": 0.0,
        "nov_epsilon_rust": 1.0e-10,
        "nov_epsilon_glsl": 10.0e-10,
        "expect": "finite",
    }


def pcg32_kat() -> dict:
    return {
        "source": "PCG32 (O'Neill 2014) demo: pcg32_srandom_r(&rng, 42u, 54u), then pcg32_random_r",
        "seed": 42,
        "seq": 54,
        "outputs": [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E],
    }


def small_case():
    import __graft_entry__

    __graft_entry__.load_package()
    from rtgallery import scenes
    from oracle.oracle import OracleScene

    sc = scenes.scene_small(64, 32)
    o = OracleScene(sc)
    # camera rays of a 32x32 grid through the scene's own camera + random rays
    rng = scenes.Pcg32(2024, 9)
    n_rand = 1024
    rays = np.zeros(2048, scenes.abi.RAY_DTYPE)
    u = rng.uniform_array(n_rand * 6).reshape(n_rand, 6)
    rays["origin"][:n_rand] = ((u[:, :3] - 0.5) * np.array([14, 3, 14]) + np.array([0, 0.6, 0])).astype(np.float32)
    d = u[:, 3:] - 0.5
    rays["direction"][:n_rand] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays["tmin"][:n_rand] = 0.0
    rays["tmax"][:n_rand] = 100.0
    eye = np.array([0, 6, -12], np.float32)
    ys, xs = np.mgrid[0:32, 0:32]
    tgt = np.stack([(xs.ravel() - 15.5) * 0.4, np.zeros(1024) - 0.35, (ys.ravel() - 15.5) * 0.4], 1)
    dd = tgt - eye
    rays["origin"][n_rand:] = eye
    rays["direction"][n_rand:] = (dd / np.linalg.norm(dd, axis=1, keepdims=True)).astype(np.float32)
    rays["tmin"][n_rand:] = 0.01
    rays["tmax"][n_rand:] = 1e4
    hits, _ = o.trace(rays)
    m0, m1 = sc.models
    return dict(
        torus_positions=m0.positions, torus_normals=m0.normals, torus_uvs=m0.uvs, torus_indices=m0.geometries[0].indices,
        ground_positions=m1.positions, ground_normals=m1.normals, ground_uvs=m1.uvs,
        ground_indices=m1.geometries[0].indices, instances=sc.instances, rays=rays, hits=hits,
    )


def main() -> None:
    (HERE / "ggx_division_by_zero.json").write_text(json.dumps(ggx_kat(), indent=1) + "\n")
    (HERE / "pcg32_kat.json").write_text(json.dumps(pcg32_kat(), indent=1) + "\n")
    np.savez_compressed(HERE / "small_rays.npz", **small_case())
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
