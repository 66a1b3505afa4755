"""ctypes wrapper of the CPU oracle (liboracle.so).  TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this
module.  It restates the reference's shader logic (see rt_oracle.c) over its
own binary SAH BVH; the product library never calls it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIB = None


class OGeometry(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("stride_floats", C.c_uint32), ("max_vertex", C.c_uint32),
                ("indices", C.c_void_p), ("primitive_count", C.c_uint32), ("flags", C.c_uint32)]


class OGeometryInfo(C.Structure):
    _fields_ = [("indices", C.c_void_p), ("diffuse_image_index", C.c_uint32),
                ("metallic_roughness_image_index", C.c_uint32), ("normal_map_image_index", C.c_int32),
                ("_padding", C.c_uint32)]


class OModelInfo(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p),
                ("geometries", C.POINTER(OGeometryInfo)), ("geometry_count", C.c_uint32), ("_padding", C.c_uint32)]


class OTexture(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("row_pitch", C.c_uint32),
                ("format", C.c_uint32), ("filter", C.c_uint32), ("_padding", C.c_uint32)]


class ORenderDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("max_trace_depth", C.c_uint32),
                ("shadow_ray_count", C.c_uint32), ("flags", C.c_uint32), ("row_begin", C.c_uint32),
                ("row_end", C.c_uint32), ("double_shading", C.c_uint32)]


class OStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("traversals", "primary_rays", "secondary_rays", "shadow_rays",
                                          "nodes_visited", "triangles_tested", "instances_visited")]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance_id", "<u4"),
                      ("instance_custom_index", "<u4"), ("geometry_index", "<u4"), ("primitive_index", "<u4"),
                      ("hit_kind", "<u4")])


class OHitGroup(C.Structure):
    _fields_ = [("closest_hit", C.c_uint32), ("any_hit", C.c_uint32)]


class OShaderBindingTable(C.Structure):
    _fields_ = [("hit_group_count", C.c_uint32), ("_padding", C.c_uint32), ("hit_groups", OHitGroup * 8)]


def reference_sbt() -> OShaderBindingTable:
    """src/main.rs:289-305: textured / mirror / portal closest-hits, each with
    the alpha-clip any-hit."""
    s = OShaderBindingTable()
    s.hit_group_count = 3
    for i, prog in enumerate((1, 2, 3)):
        s.hit_groups[i].closest_hit = prog
        s.hit_groups[i].any_hit = 1
    return s


def load() -> C.CDLL:
    global _LIB
    if _LIB is None:
        lib = C.CDLL(str(_build.build()))
        lib.o_scene_create.restype = C.c_void_p
        lib.o_scene_destroy.argtypes = [C.c_void_p]
        lib.o_scene_add_blas.argtypes = [C.c_void_p, C.POINTER(OGeometry), C.c_uint32]
        lib.o_scene_set_instances.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        lib.o_scene_set_models.argtypes = [C.c_void_p, C.POINTER(OModelInfo), C.c_uint32]
        lib.o_scene_set_texture.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(OTexture)]
        lib.o_scene_build.argtypes = [C.c_void_p]
        lib.o_scene_set_bruteforce.argtypes = [C.c_void_p, C.c_int32]
        lib.o_trace_ray_buffer.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32,
                                           C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32, C.POINTER(OStats)]
        lib.o_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(ORenderDesc), C.c_void_p,
                                 C.c_void_p, C.c_int32, C.POINTER(OStats)]
        lib.o_debug_eval.argtypes = [C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int32]
        lib.o_instance_world_to_object.argtypes = [C.c_void_p, C.c_void_p]
        lib.o_sincos_f.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        _LIB = lib
    return _LIB


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class OracleScene:
    """A scene (rtgallery.scenes.Scene) loaded into the oracle."""

    def __init__(self, scene, bruteforce: bool = False):
        self.lib = load()
        self.scene = scene
        self._keep = []
        self.h = self.lib.o_scene_create()
        for m in scene.models:
            pos = np.ascontiguousarray(m.positions, np.float32)
            self._keep.append(pos)
            geoms = (OGeometry * max(len(m.geometries), 1))()
            for i, g in enumerate(m.geometries):
                idx = np.ascontiguousarray(g.indices, np.uint32)
                self._keep.append(idx)
                geoms[i].positions = _ptr(pos)
                geoms[i].stride_floats = 3
                geoms[i].max_vertex = max(len(pos) - 1, 0)
                geoms[i].indices = _ptr(idx)
                geoms[i].primitive_count = len(idx)
                geoms[i].flags = 1 if g.opaque else 0
            self.lib.o_scene_add_blas(self.h, geoms, len(m.geometries))
        self._models = (OModelInfo * max(len(scene.models), 1))()
        for i, m in enumerate(scene.models):
            pos = np.ascontiguousarray(m.positions, np.float32)
            nrm = np.ascontiguousarray(m.normals, np.float32)
            uv = np.ascontiguousarray(m.uvs, np.float32)
            gis = (OGeometryInfo * max(len(m.geometries), 1))()
            for j, g in enumerate(m.geometries):
                idx = np.ascontiguousarray(g.indices, np.uint32)
                self._keep.append(idx)
                gis[j].indices = _ptr(idx)
                gis[j].diffuse_image_index = g.diffuse_image
                gis[j].metallic_roughness_image_index = g.metallic_roughness_image
                gis[j].normal_map_image_index = g.normal_map_image
            self._keep += [pos, nrm, uv, gis]
            self._models[i].positions = _ptr(pos)
            self._models[i].normals = _ptr(nrm)
            self._models[i].uvs = _ptr(uv)
            self._models[i].geometries = gis
            self._models[i].geometry_count = len(m.geometries)
        self.lib.o_scene_set_models(self.h, self._models, len(scene.models))
        for idx, tex in scene.textures.items():
            texels = np.ascontiguousarray(tex.texels)
            self._keep.append(texels)
            t = OTexture(_ptr(texels), texels.shape[1], texels.shape[0], tex.row_pitch, tex.format, tex.filter, 0)
            self.lib.o_scene_set_texture(self.h, idx, C.byref(t))
        self.set_instances(scene.instances)
        if bruteforce:
            self.lib.o_scene_set_bruteforce(self.h, 1)

    def set_instances(self, instances: np.ndarray) -> None:
        inst = np.ascontiguousarray(instances)
        self._inst = inst
        self.lib.o_scene_set_instances(self.h, _ptr(inst), len(inst))
        self.lib.o_scene_build(self.h)

    def trace(self, rays: np.ndarray, ray_flags: int = 0, cull_mask: int = 0xFF, sbt_offset: int = 0, sbt=None,
              with_models: bool = True, threads: int | None = None):
        """One traceRay per ray (RtRay records); returns (RtHit records, stats)."""
        table = sbt if sbt is not None else reference_sbt()
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(len(rays), HIT_DTYPE)
        st = OStats()
        self.lib.o_trace_ray_buffer(self.h, C.addressof(table), 1 if with_models else 0, ray_flags, cull_mask,
                                    sbt_offset, _ptr(rays), len(rays), _ptr(hits), threads or default_threads(),
                                    C.byref(st))
        return hits, st.as_dict()

    def render(self, uniforms=None, width: int | None = None, height: int | None = None,
               max_trace_depth: int | None = None, shadow_ray_count: int | None = None, flags: int = 0,
               rows: tuple[int, int] | None = None, double: bool = False, threads: int | None = None, sbt=None):
        sc = self.scene
        w = width or sc.width
        h = height or sc.height
        d = ORenderDesc(w, h, max_trace_depth or sc.max_trace_depth,
                        sc.shadow_ray_count if shadow_ray_count is None else shadow_ray_count, flags,
                        rows[0] if rows else 0, rows[1] if rows else h, 1 if double else 0)
        image = np.zeros((h, w, 4), np.uint8)
        radiance = np.zeros((h, w, 4), np.float32)
        st = OStats()
        u = uniforms if uniforms is not None else sc.uniforms
        s = sbt if sbt is not None else sc.sbt
        self.lib.o_render(self.h, C.addressof(u), C.addressof(s) if s is not None else None, C.byref(d),
                          _ptr(image), _ptr(radiance), threads or default_threads(), C.byref(st))
        return image, radiance, st.as_dict()

    def close(self) -> None:
        if self.h:
            self.lib.o_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def debug_eval(fn: int, inputs: np.ndarray, count: int, out_stride: int, dbl: bool = False) -> np.ndarray:
    lib = load()
    inp = np.ascontiguousarray(inputs, np.float32)
    out = np.zeros(count * out_stride, np.float32)
    r = lib.o_debug_eval(fn, _ptr(inp), _ptr(out), count, 1 if dbl else 0)
    if r != 0:
        raise ValueError(f"o_debug_eval({fn}) failed: {r}")
    return out


def world_to_object(m: np.ndarray) -> tuple[np.ndarray, bool]:
    lib = load()
    a = np.ascontiguousarray(m, np.float32).reshape(12)
    out = np.zeros(12, np.float32)
    ok = lib.o_instance_world_to_object(_ptr(a), _ptr(out))
    return out, bool(ok)
