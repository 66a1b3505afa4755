"""The 14-DOP in a BLAS header (its corners cut instance boxes in TLAS builds).

The builder projects every triangle vertex on the seven 14-DOP axes (x, y,
z and the four diagonals), rounding each projection outward, and writes the
corners of the resulting polytope into the header (`k_dop_vertices`: every
triple of the 14 planes solved in double, points outside a plane dropped,
near-duplicates merged).  For the parity scenes' models and a displaced
icosphere this file checks, against a float64 recomputation from the mesh
on the host:
- the corners span the mesh on every axis: their largest / smallest
  projection matches the mesh's within float rounding, so no instance box
  cut to them can lose a triangle;
- every corner lies inside the mesh's 14 planes (within rounding);
- the corner set equals the host's corner set within 1e-5 of the scale.
"""
import itertools

import numpy as np
import pytest

from rtgallery import scenes

pytestmark = pytest.mark.gpu

AXES = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1], [1, 1, -1], [1, -1, 1], [-1, 1, 1]], np.float64)


def _host():
    from rtgallery import host

    return host


def _header_dop(gpu_model):
    hb = gpu_model.blas.buffer[:512].cpu().numpy()
    count = int(hb[128:132].view(np.uint32)[0])  # AsHeader.dop_count
    return hb[144:144 + 12 * count].view(np.float32).reshape(-1, 3).astype(np.float64)  # AsHeader.dop_vertex


def _mesh_vertices(model):
    used = np.unique(np.concatenate([g.indices.reshape(-1) for g in model.geometries]))
    return model.positions[used].astype(np.float64)


def _host_corners(hi, lo):
    planes = np.concatenate([AXES, -AXES])
    offs = np.concatenate([hi, -lo])
    scale = max(np.abs(offs).max(), 1e-30)
    pts = []
    for a, b, c in itertools.combinations(range(14), 3):
        m = planes[[a, b, c]]
        if abs(np.linalg.det(m)) < 1e-9:
            continue
        p = np.linalg.solve(m, offs[[a, b, c]])
        if np.all(planes @ p <= offs + 1e-9 * scale):
            pts.append(p)
    out = []
    for p in pts:
        if not any(np.all(np.abs(p - q) <= 1e-7 * scale) for q in out):
            out.append(p)
    return np.array(out), scale


def _check(model, gm, what):
    v = _mesh_vertices(model)
    proj = v @ AXES.T
    hi, lo = proj.max(axis=0), proj.min(axis=0)
    dop = _header_dop(gm)
    assert 4 <= len(dop) <= 24, (what, len(dop))
    scale = max(np.abs(hi).max(), np.abs(lo).max(), 1e-30)
    tol = 1e-5 * scale
    dproj = dop @ AXES.T
    # spans the mesh on every axis, and lies inside its planes
    assert np.all(dproj.max(axis=0) >= hi - tol) and np.all(dproj.min(axis=0) <= lo + tol), what
    assert np.all(dproj <= hi + tol) and np.all(dproj >= lo - tol), what
    # the same corners as the host's float64 construction
    corners, _ = _host_corners(hi, lo)
    d1 = np.abs(dop[:, None, :] - corners[None, :, :]).max(axis=2).min(axis=1).max()
    d2 = np.abs(corners[:, None, :] - dop[None, :, :]).max(axis=2).min(axis=1).max()
    assert max(d1, d2) <= tol, (what, d1, d2, tol)


@pytest.mark.parametrize("name", ["small", "gallery", "full"])
def test_dop_corners_of_scene_models(device, name):
    sc = {"small": lambda: scenes.scene_small(32, 32), "gallery": lambda: scenes.scene_gallery(32, 32),
          "full": lambda: scenes.scene_full(0, 16, 16)}[name]()
    gs = _host().GpuScene(device, sc)
    for k, (model, gm) in enumerate(zip(sc.models, gs.models)):
        _check(model, gm, f"{name} model {k}")


def test_dop_corners_of_displaced_icosphere(device):
    m = scenes.precision_mesh(level=5)
    gs = _host().GpuScene(device, scenes.single_mesh_scene(m))
    _check(m, gs.models[0], "icosphere level 5")
