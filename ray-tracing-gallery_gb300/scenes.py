"""Procedural scenes, cameras and uniforms for the ray-tracing core.

All inputs are generated from seeds: there is no asset loading on the hot
path's benchmark scenes.  The data model mirrors the reference's host side:

* ``Model`` = ``ModelArrays`` + per-material geometries
  (src/util_structs.rs:903-909, 1113-1137): one position / normal / uv array
  and one index list per geometry; one BLAS per model; the model's index in
  ``Scene.models`` is its ``ModelInfo`` slot (the instance custom index).
* ``Texture`` = an entry of the bindless ``textures[]`` array
  (ImageManager, src/util_structs.rs:1296-1377).
* instance records are ``VkAccelerationStructureInstanceKHR`` (64 B,
  src/gpu_structs.rs:20-58); in a ``Scene`` their BLAS field holds the model
  index, which the device host and the oracle each map to their own BLAS.

Random numbers come from PCG32 (O'Neill 2014) with explicit seeds.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

# ---------------------------------------------------------------------------
# PCG32
# ---------------------------------------------------------------------------
_MULT = 6364136223846793005
_M64 = (1 << 64) - 1


class Pcg32:
    """PCG-XSH-RR 64/32, seeded like pcg32_srandom_r(initstate, initseq)."""

    def __init__(self, seed: int, seq: int = 0xDA3E39CB94B95BDB):
        self.inc = ((seq << 1) | 1) & _M64
        self.state = 0
        self.next_u32()
        self.state = (self.state + (seed & _M64)) & _M64
        self.next_u32()

    def next_u32(self) -> int:
        old = self.state
        self.state = (old * _MULT + self.inc) & _M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self) -> float:
        """[0, 1) with 24 random bits."""
        return (self.next_u32() >> 8) * (1.0 / 16777216.0)

    def uniform_range(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.uniform()

    def u32_array(self, n: int) -> np.ndarray:
        """The next n outputs, vectorised by jumping the LCG in blocks."""
        if n <= 0:
            return np.zeros(0, np.uint32)
        block = min(n, 1 << 16)
        a = np.empty(block, np.uint64)
        c = np.empty(block, np.uint64)
        am, cm = 1, 0
        for k in range(block):
            a[k] = am
            c[k] = cm
            cm = (cm * _MULT + self.inc) & _M64
            am = (am * _MULT) & _M64
        jump_a, jump_c = np.uint64(am), np.uint64(cm)
        out = np.empty(n, np.uint32)
        s = np.uint64(self.state)
        pos = 0
        with np.errstate(over="ignore"):
            while pos < n:
                m = min(block, n - pos)
                old = a[:m] * s + c[:m]
                xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)) & np.uint64(0xFFFFFFFF)
                rot = old >> np.uint64(59)
                left = (np.uint64(32) - rot) & np.uint64(31)
                v = ((xs >> rot) | (xs << left)) & np.uint64(0xFFFFFFFF)
                out[pos:pos + m] = v.astype(np.uint32)
                pos += m
                s = jump_a * s + jump_c if m == block else a[m] * s + c[m]
        self.state = int(s)
        return out

    def uniform_array(self, n: int) -> np.ndarray:
        return ((self.u32_array(n) >> 8).astype(np.float64) * (1.0 / 16777216.0))


# ---------------------------------------------------------------------------
# Data model
# ---------------------------------------------------------------------------
@dataclass
class Geometry:
    indices: np.ndarray                 # (T, 3) uint32
    opaque: bool = True
    diffuse_image: int = 0
    metallic_roughness_image: int = 0
    normal_map_image: int = -1


@dataclass
class Model:
    positions: np.ndarray               # (V, 3) float32
    normals: np.ndarray                 # (V, 3) float32
    uvs: np.ndarray                     # (V, 2) float32
    geometries: list[Geometry]
    name: str = "model"

    @property
    def triangle_count(self) -> int:
        return sum(len(g.indices) for g in self.geometries)


@dataclass
class Texture:
    texels: np.ndarray                  # (H, W, 4) uint8 or float32
    format: int
    filter: int = abi.RT_FILTER_NEAREST

    @property
    def row_pitch(self) -> int:
        return self.texels.shape[1] * self.texels.itemsize * 4


@dataclass
class Scene:
    models: list[Model]
    textures: dict[int, Texture]
    instances: np.ndarray               # INSTANCE_DTYPE; .blas = model index
    uniforms: abi.RtUniforms
    width: int
    height: int
    max_trace_depth: int = 3
    shadow_ray_count: int = 2
    sbt: abi.RtShaderBindingTable | None = None
    name: str = "scene"
    extra: dict = field(default_factory=dict)

    @property
    def instanced_triangles(self) -> int:
        return int(sum(self.models[int(b)].triangle_count for b in self.instances["blas"]))


# ---------------------------------------------------------------------------
# Meshes
# ---------------------------------------------------------------------------
def _grid_indices(nu: int, nv: int) -> np.ndarray:
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * (nv + 1) + j
    b = (i + 1) * (nv + 1) + j
    c = b + 1
    d = a + 1
    t0 = np.stack([a, b, c], -1).reshape(-1, 3)
    t1 = np.stack([a, c, d], -1).reshape(-1, 3)
    return np.stack([t0, t1], 1).reshape(-1, 3).astype(np.uint32)


def torus(R: float = 1.0, r: float = 0.35, nu: int = 64, nv: int = 32):
    """Torus around +Y: 2*nu*nv triangles; uv in [0, 1]."""
    u = np.arange(nu + 1) / nu
    v = np.arange(nv + 1) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    phi, th = 2 * np.pi * U, 2 * np.pi * V
    ring = R + r * np.cos(th)
    pos = np.stack([ring * np.cos(phi), r * np.sin(th), ring * np.sin(phi)], -1).reshape(-1, 3)
    nrm = np.stack([np.cos(th) * np.cos(phi), np.sin(th), np.cos(th) * np.sin(phi)], -1).reshape(-1, 3)
    uv = np.stack([U, V], -1).reshape(-1, 2)
    return pos.astype(np.float32), nrm.astype(np.float32), uv.astype(np.float32), _grid_indices(nu, nv)


def _hash3(ix, iy, iz, seed: int) -> np.ndarray:
    """Integer lattice hash -> [0, 1) (PCG-RXS-M-XS 32 on a mixed key)."""
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) ^ \
            (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B9 & 0xFFFFFFFF)
        h = h * np.uint32(747796405) + np.uint32(2891336453)
        w = ((h >> ((h >> np.uint32(28)) + np.uint32(4))) ^ h) * np.uint32(277803737)
        w = (w >> np.uint32(22)) ^ w
    return w.astype(np.float64) / 4294967296.0


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Trilinear value noise in [-1, 1] with a smoothstep fade."""
    q = np.floor(p)
    f = p - q
    f = f * f * (3 - 2 * f)
    i = q.astype(np.int64)
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
                out = out + w * _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
    return 2.0 * out - 1.0


def fbm(p: np.ndarray, seed: int, octaves: int = 6) -> np.ndarray:
    total = np.zeros(len(p))
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        total += amp * value_noise(p * (2.0 ** o), seed + 7919 * o)
        norm += amp
        amp *= 0.5
    return total / norm


def _vertex_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    p = pos.astype(np.float64)
    fn = np.cross(p[idx[:, 1]] - p[idx[:, 0]], p[idx[:, 2]] - p[idx[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        for c in range(3):
            n[:, c] += np.bincount(idx[:, k], weights=fn[:, c], minlength=len(p))
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return (n / ln).astype(np.float32)


def uv_sphere(nu: int = 128, nv: int = 64, radius: float = 1.0, displacement: float = 0.05, seed: int = 0):
    """UV sphere with radial displacement `displacement * noise(seed)`."""
    u = np.arange(nu + 1) / nu
    v = np.arange(nv + 1) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    phi, th = 2 * np.pi * U, np.pi * V
    d = np.stack([np.sin(th) * np.cos(phi), np.cos(th), np.sin(th) * np.sin(phi)], -1).reshape(-1, 3)
    rr = radius * (1.0 + displacement * value_noise(d * 3.0 + 11.0, seed))
    pos = (d * rr[:, None]).astype(np.float32)
    idx = _grid_indices(nu, nv)
    nrm = _vertex_normals(pos, idx)
    uv = np.stack([U, V], -1).reshape(-1, 2).astype(np.float32)
    return pos, nrm, uv, idx


def quad_grid(nx: int, ny: int, width: float, height: float, u_repeat: float, v_repeat: float):
    """An nx*ny quad grid in the XY plane (x centred, y from 0), normal -Z."""
    x = (np.arange(nx + 1) / nx - 0.5) * width
    y = np.arange(ny + 1) / ny * height
    X, Y = np.meshgrid(x, y, indexing="ij")
    pos = np.stack([X, Y, np.zeros_like(X)], -1).reshape(-1, 3).astype(np.float32)
    nrm = np.tile(np.array([[0.0, 0.0, -1.0]], np.float32), (len(pos), 1))
    U, V = np.meshgrid(np.arange(nx + 1) / nx * u_repeat, np.arange(ny + 1) / ny * v_repeat, indexing="ij")
    uv = np.stack([U, V], -1).reshape(-1, 2).astype(np.float32)
    return pos, nrm, uv, _grid_indices(nx, ny)


def ground_plane(size: float, y: float):
    h = size / 2
    pos = np.array([[-h, y, -h], [h, y, -h], [h, y, h], [-h, y, h]], np.float32)
    nrm = np.tile(np.array([[0.0, 1.0, 0.0]], np.float32), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    return pos, nrm, uv, idx


def icosphere_bisected(level: int = 9, radius: float = 10.0, amplitude: float = 0.5, seed: int = 3,
                       octaves: int = 6):
    """Level-`level` icosphere (20*4^level faces) displaced by
    `amplitude * fbm(seed, octaves)`, then every triangle bisected at the
    midpoint of its longest edge: 2*20*4^level triangles (10,485,760 at
    level 9).  Midpoints are averages of the displaced endpoints, so the
    surface is unchanged and shared long edges share their midpoint."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * len(V) + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // len(V), uk % len(V)
        mid = V[a] + V[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = (len(V) + inv).reshape(3, -1)
        V = np.concatenate([V, mid])
        f0, f1, f2 = F[:, 0], F[:, 1], F[:, 2]
        m01, m12, m20 = m[0], m[1], m[2]
        F = np.concatenate([np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
                            np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    P = V * (radius + amplitude * fbm(V * 2.0 + 5.0, seed, octaves))[:, None]
    # bisect on the longest edge
    pa, pb, pc = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    l0 = ((pa - pb) ** 2).sum(1)
    l1 = ((pb - pc) ** 2).sum(1)
    l2 = ((pc - pa) ** 2).sum(1)
    which = np.argmax(np.stack([l0, l1, l2], 1), 1)
    rot = np.stack([F[np.arange(len(F)), which], F[np.arange(len(F)), (which + 1) % 3],
                    F[np.arange(len(F)), (which + 2) % 3]], 1)  # longest edge = (rot0, rot1)
    e = np.sort(rot[:, :2], axis=1)
    key = e[:, 0] * len(P) + e[:, 1]
    uk, inv = np.unique(key, return_inverse=True)
    mid = 0.5 * (P[uk // len(P)] + P[uk % len(P)])
    mi = len(P) + inv
    P = np.concatenate([P, mid])
    Fo = np.concatenate([np.stack([rot[:, 0], mi, rot[:, 2]], 1), np.stack([mi, rot[:, 1], rot[:, 2]], 1)])
    pos = P.astype(np.float32)
    nrm = (P / np.linalg.norm(P, axis=1, keepdims=True)).astype(np.float32)
    uv = np.zeros((len(P), 2), np.float32)
    return pos, nrm, uv, Fo.astype(np.uint32)


# ---------------------------------------------------------------------------
# Textures
# ---------------------------------------------------------------------------
def solid_rgba32f(rgba) -> Texture:
    """The reference's single-colour fallback image (R32G32B32A32_SFLOAT,
    src/util_functions.rs:204-237)."""
    return Texture(np.array(rgba, np.float32).reshape(1, 1, 4), abi.RT_FORMAT_R32G32B32A32_SFLOAT)


def metallic_roughness(metallic: float, roughness: float) -> Texture:
    """metallic_roughness_to_rgba (src/util_structs.rs:1027-1029): [1, r, m, 1]."""
    return solid_rgba32f([1.0, roughness, metallic, 1.0])


def checker_alpha_rgba8(size: int = 64, cell: int = 8, rgb=(200, 180, 90)) -> Texture:
    y, x = np.mgrid[0:size, 0:size]
    a = (((x // cell) + (y // cell)) % 2 == 0).astype(np.uint8) * 255
    t = np.zeros((size, size, 4), np.uint8)
    t[..., 0], t[..., 1], t[..., 2] = rgb
    t[..., 3] = a
    return Texture(t, abi.RT_FORMAT_R8G8B8A8_SRGB, abi.RT_FILTER_LINEAR)


def bump_normal_map_rgba8(seed: int, size: int = 64, strength: float = 0.6) -> Texture:
    """A tangent-space normal map (RGBA8 UNORM, n * 0.5 + 0.5 per channel, as
    glTF normal textures are stored) of a height field of random sinusoidal
    bumps; bilinear filtering."""
    rng = Pcg32(seed, 0x4E)
    y, x = np.mgrid[0:size, 0:size].astype(np.float64) / size
    dx = np.zeros_like(x)
    dy = np.zeros_like(y)
    for _ in range(4):
        fx, fy = 1 + int(rng.next_u32() % 4), 1 + int(rng.next_u32() % 4)
        px, py = rng.uniform() * 2 * np.pi, rng.uniform() * 2 * np.pi
        # height sin(2 pi fx x + px) * sin(2 pi fy y + py): its slopes
        dx += fx * np.cos(2 * np.pi * fx * x + px) * np.sin(2 * np.pi * fy * y + py)
        dy += fy * np.sin(2 * np.pi * fx * x + px) * np.cos(2 * np.pi * fy * y + py)
    n = np.stack([-strength * dx / 4, -strength * dy / 4, np.ones_like(x)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    t = np.zeros((size, size, 4), np.uint8)
    t[..., :3] = np.clip(np.round((n * 0.5 + 0.5) * 255), 0, 255).astype(np.uint8)
    t[..., 3] = 255
    return Texture(t, abi.RT_FORMAT_R8G8B8A8_UNORM, abi.RT_FILTER_LINEAR)


def rank_noise_rgba8(seed: int, size: int = 64) -> Texture:
    """size*size noise whose values are a random permutation of ranks
    (uniform histogram), UNORM like the reference's blue noise
    (src/main.rs:440-447)."""
    rng = Pcg32(seed, 0x51)
    keys = rng.u32_array(size * size)
    order = np.argsort(keys, kind="stable")
    rank = np.empty(size * size, np.int64)
    rank[order] = np.arange(size * size)
    v = (rank * 256 // (size * size)).astype(np.uint8).reshape(size, size)
    t = np.zeros((size, size, 4), np.uint8)
    t[..., 0] = t[..., 1] = t[..., 2] = v
    t[..., 3] = 255
    return Texture(t, abi.RT_FORMAT_R8G8B8A8_UNORM, abi.RT_FILTER_NEAREST)


# ---------------------------------------------------------------------------
# Camera, projection, uniforms, instances
# ---------------------------------------------------------------------------
def look_at_view_inverse(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera-to-world (the inverse view matrix), column-major 4x4 float32.
    View space is right-handed: +X right, +Y up, the camera looks down -Z."""
    eye, target, up = (np.asarray(a, np.float64) for a in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, u, -f, eye
    return m.T.reshape(-1).astype(np.float32)  # column-major flattening


def perspective_reversed_infinite_z_vk_inverse(fovy: float, aspect: float, near: float) -> np.ndarray:
    """Inverse of the Vulkan reversed-infinite-Z projection used at
    src/main.rs:586-593 (clip = (sx x, -sy y, near, -z), sy = 1/tan(fovy/2),
    sx = sy/aspect), column-major float32."""
    sy = 1.0 / math.tan(fovy / 2.0)
    sx = sy / aspect
    cols = [[1.0 / sx, 0, 0, 0], [0, -1.0 / sy, 0, 0], [0, 0, 0, 1.0 / near], [0, 0, -1.0, 0]]
    return np.array(cols, np.float64).reshape(-1).astype(np.float32)


def make_uniforms(view_inverse, proj_inverse, sun_dir, sun_radius: float, blue_noise_index: int,
                  ggx_lut_index: int, frame_index: int = 0, show_heatmap: bool = False) -> abi.RtUniforms:
    u = abi.RtUniforms()
    for i in range(16):
        u.view_inverse[i] = float(view_inverse[i])
        u.proj_inverse[i] = float(proj_inverse[i])
    sd = np.asarray(sun_dir, np.float64)
    sd = (sd / np.linalg.norm(sd)).astype(np.float32)
    for i in range(3):
        u.sun_dir[i] = float(sd[i])
    u.sun_radius = float(np.float32(sun_radius))
    u.blue_noise_texture_index = blue_noise_index
    u.ggx_lut_texture_index = ggx_lut_index
    u.frame_index = frame_index
    u.show_heatmap = 1 if show_heatmap else 0
    return u


def instance_records(transforms: np.ndarray, model_index, custom_index, sbt_offset, flags=0,
                     mask: int = 0xFF) -> np.ndarray:
    """Packs VkAccelerationStructureInstanceKHR records (src/gpu_structs.rs:27-53):
    custom index | mask << 24, SBT offset | flags << 24, BLAS (= model index)."""
    n = len(transforms)
    out = np.zeros(n, abi.INSTANCE_DTYPE)
    out["transform"] = np.asarray(transforms, np.float32).reshape(n, 3, 4)
    ci = np.broadcast_to(np.asarray(custom_index, np.uint64), (n,))
    so = np.broadcast_to(np.asarray(sbt_offset, np.uint64), (n,))
    fl = np.broadcast_to(np.asarray(flags, np.uint64), (n,))
    out["custom_index_and_mask"] = ((ci & 0xFFFFFF) | (np.uint64(mask) << np.uint64(24))).astype(np.uint32)
    out["sbt_offset_and_flags"] = ((so & 0xFFFFFF) | ((fl & 0xFF) << np.uint64(24))).astype(np.uint32)
    out["blas"] = np.broadcast_to(np.asarray(model_index, np.uint64), (n,))
    return out


def rot_y(a: float) -> np.ndarray:
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def affine(rot: np.ndarray, t, scale: float = 1.0) -> np.ndarray:
    m = np.zeros((3, 4))
    m[:, :3] = rot * scale
    m[:, 3] = t
    return m


def random_rotation(rng: Pcg32) -> np.ndarray:
    """Uniform on SO(3) from a uniform unit quaternion (Shoemake 1992)."""
    u1, u2, u3 = rng.uniform(), rng.uniform(), rng.uniform()
    a, b = math.sqrt(1 - u1), math.sqrt(u1)
    x, y = a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2)
    z, w = b * math.sin(2 * math.pi * u3), b * math.cos(2 * math.pi * u3)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _model(arrays, name, geoms) -> Model:
    pos, nrm, uv, idx = arrays
    return Model(pos, nrm, uv, geoms(idx), name)


# ---------------------------------------------------------------------------
# Benchmark scenes
# ---------------------------------------------------------------------------
TEX_DIFFUSE_A = 0
TEX_DIFFUSE_B = 1
TEX_BLUE_NOISE = 2      # as the reference (src/main.rs:594)
TEX_GGX_LUT = 3         # as the reference (src/main.rs:595); brdf never samples it
TEX_MR_DEFAULT = 4
TEX_FENCE = 5
TEX_MR_SHINY = 6
TEX_MIRROR_TINT = 7
TEX_NORMAL_MAP = 8


def _base_textures(seed: int) -> dict[int, Texture]:
    return {
        TEX_DIFFUSE_A: solid_rgba32f([0.8, 0.55, 0.3, 1.0]),
        TEX_DIFFUSE_B: solid_rgba32f([0.45, 0.5, 0.55, 1.0]),
        TEX_BLUE_NOISE: rank_noise_rgba8(seed),
        TEX_GGX_LUT: solid_rgba32f([1.0, 1.0, 0.0, 1.0]),
        TEX_MR_DEFAULT: metallic_roughness(0.0, 0.6),
        TEX_FENCE: checker_alpha_rgba8(),
        TEX_MR_SHINY: metallic_roughness(0.5, 0.3),
        TEX_MIRROR_TINT: solid_rgba32f([1.0, 1.0, 1.0, 1.0]),
        TEX_NORMAL_MAP: bump_normal_map_rgba8(seed),
    }


SUN_DIR_CONFIG = (0.3, -1.0, 0.2)   # light travel direction; uniforms hold -dir


def scene_small(width: int = 256, height: int = 256, seed: int = 1) -> Scene:
    """Plain FP32 path, small: a 64x32 torus (R=1, r=0.35, 4096 tris)
    instanced 16x on a 4x4 grid (spacing 3, random Y rotation from PCG32(seed))
    over a 2-triangle 40x40 ground; pinhole camera, 60 deg FOV, at (0,6,-12)
    looking at the origin; directional light normalize(0.3,-1,0.2); 1 primary
    + 1 hard shadow per pixel (sun_radius 0); constant albedo."""
    rng = Pcg32(seed)
    tor = _model(torus(1.0, 0.35, 64, 32), "torus",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_A, TEX_MR_DEFAULT)])
    gnd = _model(ground_plane(40.0, -0.35), "ground",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_B, TEX_MR_DEFAULT)])
    xf, mdl = [], []
    for gx in range(4):
        for gz in range(4):
            xf.append(affine(rot_y(rng.uniform() * 2 * math.pi), [(gx - 1.5) * 3.0, 0.0, (gz - 1.5) * 3.0]))
            mdl.append(0)
    xf.append(affine(np.eye(3), [0, 0, 0]))
    mdl.append(1)
    inst = instance_records(np.array(xf), np.array(mdl), np.array(mdl), abi.HIT_SHADER_TEXTURED)
    u = make_uniforms(look_at_view_inverse((0, 6, -12), (0, 0, 0)),
                      perspective_reversed_infinite_z_vk_inverse(math.radians(60), width / height, 0.1),
                      -np.asarray(SUN_DIR_CONFIG), 0.0, TEX_BLUE_NOISE, TEX_GGX_LUT, 0)
    return Scene([tor, gnd], _base_textures(seed), inst, u, width, height, max_trace_depth=3, shadow_ray_count=1,
                 name="small-4x4-tori")


FULL_INSTANCES = 256
FULL_BOX = 50.0


def full_scene_models(seed: int = 7) -> list[Model]:
    tor = _model(torus(1.0, 0.35, 64, 32), "torus",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_A, TEX_MR_DEFAULT)])
    sph = _model(uv_sphere(128, 64, 1.0, 0.05, seed), "sphere",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_B, TEX_MR_SHINY)])
    fen = _model(quad_grid(200, 1, 10.0, 2.0, 25.0, 1.0), "fence",
                 lambda idx: [Geometry(idx, False, TEX_FENCE, TEX_MR_DEFAULT)])
    return [tor, sph, fen]


def full_scene_instances(frame: int, seed: int = 7, count: int = FULL_INSTANCES) -> np.ndarray:
    """Per-frame rigid transforms: rotation uniform on SO(3), translation
    uniform in a 50^3 box; each instance keeps a fixed model, scale and
    material (10% mirrors) drawn from the scene seed."""
    srng = Pcg32(seed, 0xA5)
    models, scales, sbts = [], [], []
    for i in range(count):
        models.append(int(srng.next_u32() % 3))
        scales.append(srng.uniform_range(1.5, 4.0))
        sbts.append(abi.HIT_SHADER_MIRROR if srng.uniform() < 0.1 else abi.HIT_SHADER_TEXTURED)
    frng = Pcg32(seed * 1000003 + frame, 0xF0 + frame)
    xf = []
    for i in range(count):
        r = random_rotation(frng)
        t = [frng.uniform_range(-FULL_BOX / 2, FULL_BOX / 2) for _ in range(3)]
        xf.append(affine(r, t, scales[i]))
    flags = [abi.RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE if m == 2 else 0 for m in models]
    return instance_records(np.array(xf), np.array(models), np.array(models), np.array(sbts), np.array(flags))


def scene_full(frame: int = 0, width: int = 1920, height: int = 1080, seed: int = 7,
               models: list[Model] | None = None) -> Scene:
    """Full plain feature set at 1920x1080: 256 instances of {torus 64x32,
    UV sphere 128x64 displaced by 0.05*noise(seed), alpha-clipped 200x1 quad
    fence with a 64x64 RGBA8 checker alpha (threshold 0.5)}; 10% mirrors;
    per-frame random rigid transforms driving a TLAS rebuild; 4 blue-noise
    soft-shadow rays per textured hit (light cone half-angle 2 deg, used as
    sun_radius = tan 2 deg); 1 reflection bounce (max_trace_depth 2)."""
    models = models if models is not None else full_scene_models(seed)
    inst = full_scene_instances(frame, seed)
    u = make_uniforms(look_at_view_inverse((0, 18, -62), (0, 0, 0)),
                      perspective_reversed_infinite_z_vk_inverse(math.radians(60), width / height, 0.1),
                      -np.asarray(SUN_DIR_CONFIG), math.tan(math.radians(2.0)), TEX_BLUE_NOISE, TEX_GGX_LUT, frame)
    return Scene(models, _base_textures(seed), inst, u, width, height, max_trace_depth=2, shadow_ray_count=4,
                 name="full-256-instances")


def scene_gallery(width: int = 320, height: int = 200, seed: int = 11, frame: int = 0) -> Scene:
    """A small scene that exercises every program of the reference: textured
    tori and a normal-mapped ground, mirror tori, a portal plane (SBT offset
    2) and an alpha-clipped double-sided fence, soft shadows (2 rays,
    sun_radius 0.05) and the 3-iteration bounce loop, as DefaultScene lays
    them out (src/scene.rs:95-156).  The ground's geometry names a normal map
    (closest_hit_textured.glsl:123-157: the cotangent frame from its
    positions and UVs); the tori have none."""
    rng = Pcg32(seed)
    tor = _model(torus(1.0, 0.35, 32, 16), "torus", lambda idx: [Geometry(idx, True, TEX_DIFFUSE_A, TEX_MR_SHINY)])
    pln = _model(ground_plane(2.0, 0.0), "plane",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_B, TEX_MR_DEFAULT, TEX_NORMAL_MAP)])
    fen = _model(quad_grid(20, 1, 2.0, 1.0, 4.0, 1.0), "fence",
                 lambda idx: [Geometry(idx, False, TEX_FENCE, TEX_MR_DEFAULT)])
    xf, mdl, sbt, flg = [], [], [], []

    def add(m, s, f, t):
        xf.append(t); mdl.append(m); sbt.append(s); flg.append(f)

    add(1, abi.HIT_SHADER_TEXTURED, 0, affine(np.eye(3), [0, 0, 0], 10.0))
    add(0, abi.HIT_SHADER_TEXTURED, 0, affine(np.eye(3), [0, 1, 0]))
    add(1, abi.HIT_SHADER_PORTAL, abi.RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE, affine(np.eye(3), [3.5, 1.0, 0.5]))
    add(2, abi.HIT_SHADER_TEXTURED, abi.RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE, affine(np.eye(3), [2, 0, 2]))
    for _ in range(30):
        t = [rng.uniform_range(-5, 5), rng.uniform_range(0.5, 2.5), rng.uniform_range(-5, 5)]
        r = rot_y(rng.uniform_range(0, 100))
        s = rng.uniform_range(0.2, 0.6)
        add(0, abi.HIT_SHADER_TEXTURED if rng.uniform() < 0.5 else abi.HIT_SHADER_MIRROR, 0, affine(r, t, s))
    inst = instance_records(np.array(xf), np.array(mdl), np.array(mdl), np.array(sbt), np.array(flg))
    u = make_uniforms(look_at_view_inverse((-4.0, 3.5, -7.0), (0.5, 0.8, 0.5)),
                      perspective_reversed_infinite_z_vk_inverse(math.radians(59), width / height, 0.1),
                      (0.45, 0.8, -0.4), 0.05, TEX_BLUE_NOISE, TEX_GGX_LUT, frame)
    return Scene([tor, pln, fen], _base_textures(seed), inst, u, width, height, max_trace_depth=3, shadow_ray_count=2,
                 name="gallery")


def precision_mesh(level: int = 9, seed: int = 3) -> Model:
    pos, nrm, uv, idx = icosphere_bisected(level, 10.0, 0.5, seed, 6)
    return Model(pos, nrm, uv, [Geometry(idx, True, TEX_DIFFUSE_A, TEX_MR_DEFAULT)], f"icosphere-l{level}-bisected")


def random_rays(count: int, seed: int = 5, box: float = 30.0) -> np.ndarray:
    """Origins uniform in a box^3 cube centred on the origin, directions
    uniform on S^2 (normalised Box-Muller Gaussians), tmin 0, tmax +inf."""
    rng = Pcg32(seed, 0x77)
    u = rng.uniform_array(count * 7).reshape(count, 7)
    rays = np.zeros(count, abi.RAY_DTYPE)
    rays["origin"] = ((u[:, :3] - 0.5) * box).astype(np.float32)
    r1 = np.sqrt(-2.0 * np.log(1.0 - u[:, 3:5]))
    g = np.stack([r1[:, 0] * np.cos(2 * np.pi * u[:, 5]), r1[:, 0] * np.sin(2 * np.pi * u[:, 5]),
                  r1[:, 1] * np.cos(2 * np.pi * u[:, 6])], 1)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    rays["direction"] = g.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.inf
    return rays


def single_mesh_scene(model: Model, width: int = 64, height: int = 64) -> Scene:
    inst = instance_records(affine(np.eye(3), [0, 0, 0])[None], np.array([0]), np.array([0]), 0)
    u = make_uniforms(look_at_view_inverse((0, 0, -30), (0, 0, 0)),
                      perspective_reversed_infinite_z_vk_inverse(math.radians(60), 1.0, 0.1),
                      -np.asarray(SUN_DIR_CONFIG), 0.0, TEX_BLUE_NOISE, TEX_GGX_LUT)
    return Scene([model], _base_textures(1), inst, u, width, height, name=model.name)


BATCH_RESOLUTIONS = ((128, 128), (256, 256), (512, 512), (1024, 1024), (1920, 1080))
BATCH_TRIS = (10_000, 2_000_000)


def _procedural_scene(rng: Pcg32, target: float, width: int, height: int, seed: int, name: str) -> Scene:
    """A procedural torus, a displaced UV sphere and a ground grid whose
    unique triangles total about `target` (split 1/2, 1/3, 1/6), instanced
    six, four and one times (one torus a mirror), seen from a random bearing."""

    def grid_dims(tris, aspect):
        nv = max(3, int(round(math.sqrt(tris / (2.0 * aspect)))))
        return max(3, int(round(tris / (2.0 * nv)))), nv

    tu, tv = grid_dims(target / 2, 2.0)
    su, sv = grid_dims(target / 3, 2.0)
    gx = max(1, int(round(math.sqrt(target / 12))))
    tor = _model(torus(1.0, 0.35, tu, tv), f"torus{tu}x{tv}",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_A, TEX_MR_SHINY)])
    sph = _model(uv_sphere(su, sv, 1.0, 0.05, seed), f"sphere{su}x{sv}",
                 lambda idx: [Geometry(idx, True, TEX_DIFFUSE_B, TEX_MR_DEFAULT)])
    gp, gn, guv, gi = quad_grid(gx, gx, 40.0, 40.0, 8.0, 8.0)
    rot = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]], np.float32)  # XY grid -> y = 0, normal +y
    gp = (gp @ rot.T).astype(np.float32)
    gn = (gn @ rot.T).astype(np.float32)
    grd = _model((gp, gn, guv, gi), f"ground{gx}x{gx}", lambda idx: [Geometry(idx, True, TEX_DIFFUSE_B, TEX_MR_DEFAULT)])
    xf, mdl, sbt = [affine(np.eye(3), [0.0, -1.2, -20.0])], [2], [abi.HIT_SHADER_TEXTURED]
    for k in range(10):
        t = [rng.uniform_range(-6, 6), rng.uniform_range(-0.5, 2.5), rng.uniform_range(-6, 6)]
        m = 0 if k < 6 else 1
        xf.append(affine(random_rotation(rng), t, rng.uniform_range(0.6, 1.6)))
        mdl.append(m)
        sbt.append(abi.HIT_SHADER_MIRROR if k == 0 else abi.HIT_SHADER_TEXTURED)
    inst = instance_records(np.array(xf), np.array(mdl), np.array(mdl), np.array(sbt))
    a = rng.uniform_range(0.0, 2.0 * math.pi)
    eye = (12.0 * math.cos(a), rng.uniform_range(4.0, 9.0), 12.0 * math.sin(a))
    u = make_uniforms(look_at_view_inverse(eye, (0.0, 0.5, 0.0)),
                      perspective_reversed_infinite_z_vk_inverse(math.radians(60), width / height, 0.1),
                      -np.asarray(SUN_DIR_CONFIG), math.tan(math.radians(2.0)), TEX_BLUE_NOISE, TEX_GGX_LUT, 0)
    return Scene([tor, sph, grd], _base_textures(seed), inst, u, width, height, max_trace_depth=2,
                 shadow_ray_count=2, name=name)


def scene_batch_member(index: int, seed: int = 23) -> Scene:
    """One scene of the batched workload: a procedural torus, a displaced UV
    sphere and a ground grid whose unique triangles total a log-uniform count
    in [10k, 2M] (split 1/2, 1/3, 1/6), instanced six, four and one times
    (one torus a mirror); resolution drawn from {128^2, 256^2, 512^2,
    1024^2, 1920x1080}; primary rays, 2 blue-noise soft shadows (2 deg) and
    1 reflection bounce.  Everything follows from (seed, index)."""
    rng = Pcg32(seed * 7919 + index, 0xB7 + index)
    lo, hi = math.log(BATCH_TRIS[0]), math.log(BATCH_TRIS[1])
    target = math.exp(lo + (hi - lo) * rng.uniform())
    width, height = BATCH_RESOLUTIONS[int(rng.next_u32() % len(BATCH_RESOLUTIONS))]
    sc = _procedural_scene(rng, target, width, height, seed + index, f"batch-{index}")
    sc.uniforms.frame_index = index
    return sc


def batch_scenes(count: int = 64, seed: int = 23) -> list[Scene]:
    return [scene_batch_member(i, seed) for i in range(count)]


def random_view_uniforms(rng: Pcg32, width: int, height: int, frame: int = 0, distance=(8.0, 16.0),
                         height_range=(2.0, 9.0), target=(0.0, 0.5, 0.0)) -> abi.RtUniforms:
    """A request's camera and light: eye on a random bearing around `target`,
    sun direction random above the horizon, 2 degree soft-shadow cone."""
    a = rng.uniform_range(0.0, 2.0 * math.pi)
    r = rng.uniform_range(*distance)
    eye = (target[0] + r * math.cos(a), rng.uniform_range(*height_range), target[2] + r * math.sin(a))
    sa = rng.uniform_range(0.0, 2.0 * math.pi)
    el = rng.uniform_range(0.3, 1.3)
    to_sun = np.array([math.cos(el) * math.cos(sa), math.sin(el), math.cos(el) * math.sin(sa)])
    return make_uniforms(look_at_view_inverse(eye, target),
                         perspective_reversed_infinite_z_vk_inverse(math.radians(60), width / height, 0.1),
                         to_sun, math.tan(math.radians(2.0)), TEX_BLUE_NOISE, TEX_GGX_LUT, frame)


SERVE_RESOLUTIONS = ((256, 256), (512, 512), (1024, 1024), (1280, 720), (1920, 1080))
SERVE_TRIS = (50_000, 4_000_000)


def scene_serve_member(index: int, seed: int = 31) -> Scene:
    """One resident scene of the serving workload: the batch scene's layout
    (torus, displaced sphere, ground grid) with unique triangles log-uniform
    in [50k, 4M]; camera, light, size and shadow count come per request."""
    rng = Pcg32(seed * 104729 + index, 0xC3 + index)
    lo, hi = math.log(SERVE_TRIS[0]), math.log(SERVE_TRIS[1])
    target = math.exp(lo + (hi - lo) * rng.uniform())
    sc = _procedural_scene(rng, target, 256, 256, seed + 1000 + index, f"serve-{index}")
    sc.max_trace_depth, sc.shadow_ray_count = 2, 2
    return sc
