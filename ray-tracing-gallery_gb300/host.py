"""Host side above the C ABI, mirroring the reference's Rust host for this path.

Names follow the reference so a maintainer can map each call:

=====================================  =========================================
this module                            reference (src/...)
=====================================  =========================================
ScratchBuffer.ensure_size_of           util_structs.rs:420-524 (grow-only)
AccelerationStructure.build_blas       util_structs.rs:140-224 (+ new :226-283)
AccelerationStructure.build_tlas       util_functions.rs:453-510 (build_tlas)
AccelerationStructure.update_tlas      util_structs.rs:285-357
AccelerationStructure.clone            util_structs.rs:359-405
GpuModel.new                           Model::new, util_structs.rs:1158-1236
ImageManager.push_image                util_structs.rs:1296-1377
PerFrameResources.record               command_buffer_recording.rs:79-126
=====================================  =========================================

Device memory comes from PyTorch (its caching allocator returns 512-byte
aligned blocks); every compute call goes through librtcore.so.  There is no
CPU fallback: without a CUDA device or without the built library these
classes raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .scenes import Model, Scene, Texture

try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the image
    torch = None


def _require_cuda():
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required for the ray-tracing core (there is no CPU fallback)")


class Device:
    """One librtcore context on the current CUDA device."""

    def __init__(self, threadsafe: bool = False):
        _require_cuda()
        self.lib = abi.load_library()
        torch.cuda.init()
        self.ctx = C.c_void_p()
        self.check(self.lib.rt_ctx_create(abi.RT_CTX_THREADSAFE if threadsafe else 0, C.byref(self.ctx)))
        self._texture_refs: dict[int, object] = {}

    # -- plumbing ---------------------------------------------------------
    def check(self, status: int) -> None:
        abi.check(self.lib, status)

    @staticmethod
    def stream_handle(stream=None) -> C.c_void_p:
        s = stream if stream is not None else torch.cuda.current_stream()
        return C.c_void_p(s.cuda_stream)

    @staticmethod
    def alloc(nbytes: int) -> "torch.Tensor":
        t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device="cuda")
        assert t.data_ptr() % abi.RT_AS_ALIGNMENT == 0
        return t

    @staticmethod
    def upload(a: np.ndarray) -> "torch.Tensor":
        a = np.ascontiguousarray(a)
        t = torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).to("cuda")
        return t

    @classmethod
    def texture_desc(cls, tex: Texture) -> tuple[abi.RtTextureDesc, "torch.Tensor"]:
        """Uploads a texture; returns its descriptor and the buffer to keep alive."""
        buf = cls.upload(tex.texels)
        d = abi.RtTextureDesc()
        d.address = buf.data_ptr()
        d.height, d.width = tex.texels.shape[0], tex.texels.shape[1]
        d.row_pitch = tex.row_pitch
        d.format = tex.format
        d.filter = tex.filter
        return d, buf

    def set_texture(self, index: int, tex: Texture) -> None:
        d, buf = self.texture_desc(tex)
        self.check(self.lib.rt_ctx_set_texture(self.ctx, index, C.byref(d)))
        self._texture_refs[index] = buf

    def read_stats(self, reset: bool = True, stream=None) -> dict:
        s = abi.RtStats()
        self.check(self.lib.rt_ctx_read_stats(self.ctx, C.byref(s), 1 if reset else 0, self.stream_handle(stream)))
        return s.as_dict()

    def close(self) -> None:
        if self.ctx:
            torch.cuda.synchronize()
            self.lib.rt_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ScratchBuffer:
    """Grow-only scratch (ScratchBuffer::ensure_size_of): reallocated only
    when a build needs more than it holds."""

    def __init__(self, name: str = "scratch"):
        self.name = name
        self.buffer = None

    def ensure_size_of(self, size: int) -> int:
        if self.buffer is None or self.buffer.numel() < size:
            if self.buffer is not None:
                torch.cuda.current_stream().synchronize()
            self.buffer = Device.alloc(max(size, 256))
        return self.buffer.data_ptr()

    @property
    def size(self) -> int:
        return 0 if self.buffer is None else self.buffer.numel()


@dataclass
class GeometryDesc:
    """src/util_structs.rs:123-129 (`Geometry`)."""
    position_buffer_address: int
    index_buffer_address: int
    num_indices: int
    num_vertices: int
    opaque: bool


class AccelerationStructure:
    BOTTOM_LEVEL = 0
    TOP_LEVEL = 1

    def __init__(self, buffer, size: int, flags: int, ty: int, name: str = ""):
        self.buffer = buffer
        self.size = size
        self.flags = flags
        self.ty = ty
        self.name = name

    def device_address(self, device: Device | None = None) -> int:
        return self.buffer.data_ptr()

    @staticmethod
    def _geometry_array(geometries: list[GeometryDesc]):
        arr = (abi.RtGeometryTriangles * max(len(geometries), 1))()
        for i, g in enumerate(geometries):
            arr[i].vertex_address = g.position_buffer_address
            arr[i].index_address = g.index_buffer_address
            arr[i].vertex_stride = 12
            arr[i].max_vertex = max(g.num_vertices - 1, 0)
            arr[i].primitive_count = g.num_indices // 3
            arr[i].flags = abi.RT_GEOMETRY_OPAQUE if g.opaque else 0
        return arr

    @classmethod
    def build_blas(cls, device: Device, name: str, scratch: ScratchBuffer, geometries: list[GeometryDesc],
                   flags: int = abi.RT_BUILD_PREFER_FAST_TRACE, stream=None) -> "AccelerationStructure":
        arr = cls._geometry_array(geometries)
        sizes = abi.RtBuildSizes()
        device.check(device.lib.rt_get_blas_build_sizes(arr, len(geometries), flags, C.byref(sizes)))
        scr = scratch.ensure_size_of(sizes.build_scratch_size)
        buf = Device.alloc(sizes.acceleration_structure_size)
        device.check(device.lib.rt_cmd_build_blas(device.ctx, arr, len(geometries), flags, buf.data_ptr(),
                                                  sizes.acceleration_structure_size, scr, scratch.size,
                                                  Device.stream_handle(stream)))
        return cls(buf, sizes.acceleration_structure_size, flags, cls.BOTTOM_LEVEL, name)

    def rebuild_blas(self, device: Device, scratch: ScratchBuffer, geometries: list[GeometryDesc],
                     stream=None) -> None:
        """The same BLAS built again into its own memory (same geometries and
        flags): the build's device work alone, with no upload or allocation."""
        arr = self._geometry_array(geometries)
        sizes = abi.RtBuildSizes()
        device.check(device.lib.rt_get_blas_build_sizes(arr, len(geometries), self.flags, C.byref(sizes)))
        scr = scratch.ensure_size_of(sizes.build_scratch_size)
        device.check(device.lib.rt_cmd_build_blas(device.ctx, arr, len(geometries), self.flags, self.buffer.data_ptr(),
                                                  self.size, scr, scratch.size, Device.stream_handle(stream)))

    @classmethod
    def build_tlas(cls, device: Device, instances, num_instances: int, scratch: ScratchBuffer,
                   flags: int = abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_ALLOW_UPDATE,
                   stream=None) -> "AccelerationStructure":
        sizes = abi.RtBuildSizes()
        device.check(device.lib.rt_get_tlas_build_sizes(num_instances, flags, C.byref(sizes)))
        scr = scratch.ensure_size_of(sizes.build_scratch_size)
        buf = Device.alloc(sizes.acceleration_structure_size)
        device.check(device.lib.rt_cmd_build_tlas(device.ctx, instances.data_ptr(), num_instances, flags,
                                                  buf.data_ptr(), sizes.acceleration_structure_size, scr,
                                                  scratch.size, Device.stream_handle(stream)))
        return cls(buf, sizes.acceleration_structure_size, flags, cls.TOP_LEVEL, "tlas")

    def rebuild_tlas(self, device: Device, instances, num_instances: int, scratch: ScratchBuffer, stream=None) -> None:
        """Full rebuild into the same memory (instance count unchanged)."""
        sizes = abi.RtBuildSizes()
        device.check(device.lib.rt_get_tlas_build_sizes(num_instances, self.flags, C.byref(sizes)))
        scr = scratch.ensure_size_of(sizes.build_scratch_size)
        device.check(device.lib.rt_cmd_build_tlas(device.ctx, instances.data_ptr(), num_instances, self.flags,
                                                  self.buffer.data_ptr(), self.size, scr, scratch.size,
                                                  Device.stream_handle(stream)))

    def update_tlas(self, device: Device, instances, num_instances: int, scratch: ScratchBuffer, stream=None) -> None:
        """In-place refit (src == dst), util_structs.rs:318-319."""
        sizes = abi.RtBuildSizes()
        device.check(device.lib.rt_get_tlas_build_sizes(num_instances, self.flags, C.byref(sizes)))
        scr = scratch.ensure_size_of(sizes.update_scratch_size)
        addr = self.buffer.data_ptr()
        device.check(device.lib.rt_cmd_update_tlas(device.ctx, instances.data_ptr(), num_instances, addr, addr,
                                                   self.size, scr, scratch.size, Device.stream_handle(stream)))

    def clone(self, device: Device, name: str, stream=None) -> "AccelerationStructure":
        buf = Device.alloc(self.size)
        device.check(device.lib.rt_cmd_copy_acceleration_structure(device.ctx, self.buffer.data_ptr(), buf.data_ptr(),
                                                                   self.size, abi.RT_COPY_MODE_CLONE,
                                                                   Device.stream_handle(stream)))
        return AccelerationStructure(buf, self.size, self.flags, self.ty, name)

    def info(self, device: Device, stream=None) -> abi.RtAccelerationStructureInfo:
        inf = abi.RtAccelerationStructureInfo()
        device.check(device.lib.rt_get_acceleration_structure_info(self.buffer.data_ptr(), C.byref(inf),
                                                                   Device.stream_handle(stream)))
        return inf


class GpuModel:
    """Model::new: vertex, normal, uv, index and geometry-info buffers plus
    the model's BLAS (one geometry per material)."""

    def __init__(self, device: Device, model: Model, scratch: ScratchBuffer, model_id: int,
                 build_flags: int = abi.RT_BUILD_PREFER_FAST_TRACE, stream=None):
        self.id = model_id
        self.name = model.name
        self.position_buffer = Device.upload(np.ascontiguousarray(model.positions, np.float32))
        self.normal_buffer = Device.upload(np.ascontiguousarray(model.normals, np.float32))
        self.uv_buffer = Device.upload(np.ascontiguousarray(model.uvs, np.float32))
        self.index_buffers = []
        infos = np.zeros(len(model.geometries), abi.GEOMETRY_INFO_DTYPE)
        geoms = []
        for i, g in enumerate(model.geometries):
            ib = Device.upload(np.ascontiguousarray(g.indices, np.uint32))
            self.index_buffers.append(ib)
            geoms.append(GeometryDesc(self.position_buffer.data_ptr(), ib.data_ptr(), int(g.indices.size),
                                      len(model.positions), g.opaque))
            infos[i] = (ib.data_ptr(), g.diffuse_image, g.metallic_roughness_image, g.normal_map_image, 0)
        self.geometry_info_buffer = Device.upload(infos)
        self.geometries = geoms
        self.blas = AccelerationStructure.build_blas(device, f"{model.name} blas", scratch, geoms, build_flags,
                                                     stream)

    def model_info(self) -> tuple:
        return (self.position_buffer.data_ptr(), self.normal_buffer.data_ptr(), self.uv_buffer.data_ptr(),
                self.geometry_info_buffer.data_ptr())


class ImageManager:
    """The bindless texture array: every texture of a scene bound at its index."""

    def __init__(self, device: Device):
        self.device = device

    def push_images(self, textures: dict[int, Texture]) -> None:
        for idx, tex in textures.items():
            self.device.set_texture(idx, tex)


class GpuScene:
    """Everything a scene needs resident on the device: models with BLASes,
    the ModelInfo array, textures, the instance buffer and its TLAS."""

    def __init__(self, device: Device, scene: Scene, scratch: ScratchBuffer | None = None,
                 tlas_flags: int = abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_ALLOW_UPDATE, stream=None,
                 blas_flags: int | list[int] = abi.RT_BUILD_PREFER_FAST_TRACE, own_textures: bool = False):
        """own_textures: keep the scene's bindless table in its own device array
        (for batched rendering of scenes with different textures) instead of
        binding the textures into the context's table.  blas_flags: one value
        for every model, or one per model (e.g. some quantised, some FP32)."""
        self.device = device
        self.scene = scene
        self.scratch = scratch or ScratchBuffer("scene scratch")
        per_model = blas_flags if isinstance(blas_flags, (list, tuple)) else [blas_flags] * len(scene.models)
        self.models = [GpuModel(device, m, self.scratch, i, build_flags=per_model[i], stream=stream)
                       for i, m in enumerate(scene.models)]
        infos = np.array([m.model_info() for m in self.models], abi.MODEL_INFO_DTYPE)
        self.model_info_buffer = Device.upload(infos)
        self.texture_table, self.texture_count, self._texture_refs = None, 0, []
        self.texture_descs = None
        if own_textures:
            n = max(scene.textures) + 1 if scene.textures else 1
            table = (abi.RtTextureDesc * n)()
            for idx, tex in scene.textures.items():
                table[idx], buf = Device.texture_desc(tex)
                self._texture_refs.append(buf)
            self.texture_table = Device.upload(np.frombuffer(bytes(table), np.uint8))
            self.texture_count = n
            self.texture_descs = table
        else:
            ImageManager(device).push_images(scene.textures)
        self.num_instances = len(scene.instances)
        self.instances_host = self.patch_instances(scene.instances)
        self.instances_buffer = Device.upload(self.instances_host)
        self.tlas = AccelerationStructure.build_tlas(device, self.instances_buffer, self.num_instances, self.scratch,
                                                     tlas_flags, stream)

    def bind_textures(self) -> None:
        """Binds a scene with its own texture table into the context's
        bindless table (rt_ctx_set_texture per index), as a host that renders
        several scenes through rt_cmd_trace_rays does before each call."""
        if self.texture_descs is None:
            raise ValueError("bind_textures needs a scene built with own_textures=True")
        for idx in range(self.texture_count):
            self.device.check(self.device.lib.rt_ctx_set_texture(self.device.ctx, idx,
                                                                 C.byref(self.texture_descs[idx])))

    def patch_instances(self, instances: np.ndarray) -> np.ndarray:
        """Scene instances carry model indices; replace them by BLAS addresses."""
        out = instances.copy()
        addrs = np.array([m.blas.device_address() for m in self.models], np.uint64)
        out["blas"] = addrs[instances["blas"].astype(np.int64)]
        return out

    def push_constants(self, uniforms_address: int, tlas: AccelerationStructure | None = None):
        p = abi.RtPushConstantBufferAddresses()
        p.model_info = self.model_info_buffer.data_ptr()
        p.uniforms = uniforms_address
        p.acceleration_structure = (tlas or self.tlas).device_address()
        return p


class PerFrameResources:
    """command_buffer_recording.rs:22-55: per-frame uniforms, output image,
    instance buffer and TLAS (a CLONE of the scene's, src/main.rs:600-668)."""

    def __init__(self, device: Device, gpu_scene: GpuScene, width: int, height: int, radiance: bool = False,
                 clone_tlas: bool = False):
        self.device = device
        self.gpu_scene = gpu_scene
        self.width, self.height = width, height
        self.uniforms_buffer = Device.alloc(C.sizeof(abi.RtUniforms))
        self.image = torch.zeros((height, width, 4), dtype=torch.uint8, device="cuda")
        self.radiance = torch.zeros((height, width, 4), dtype=torch.float32, device="cuda") if radiance else None
        self.instances_buffer = gpu_scene.instances_buffer.clone()
        self.num_instances = gpu_scene.num_instances
        self.scratch = ScratchBuffer("frame scratch")
        self.tlas = gpu_scene.tlas.clone(device, "frame tlas") if clone_tlas else gpu_scene.tlas

    def write_uniforms(self, uniforms: abi.RtUniforms, stream=None) -> None:
        host = torch.frombuffer(bytearray(bytes(uniforms)), dtype=torch.uint8)
        self.uniforms_buffer.copy_(host, non_blocking=False)

    def record(self, max_trace_depth: int, shadow_ray_count: int, flags: int = 0,
               sbt: abi.RtShaderBindingTable | None = None, stream=None, image_address: int | None = None) -> None:
        """cmd_trace_rays(raygen, miss, hit, {}, W, H, 1).  image_address:
        where the RGBA8 image goes instead of this frame's device image (e.g.
        a page-locked host buffer, which the GPU writes through its mapping)."""
        push = self.gpu_scene.push_constants(self.uniforms_buffer.data_ptr(), self.tlas)
        d = abi.RtTraceRaysDesc()
        d.width, d.height = self.width, self.height
        d.max_trace_depth = max_trace_depth
        d.shadow_ray_count = shadow_ray_count
        d.flags = flags
        d.image_address = image_address if image_address is not None else self.image.data_ptr()
        d.radiance_address = self.radiance.data_ptr() if self.radiance is not None else 0
        sbt_p = C.byref(sbt) if sbt is not None else None
        self.device.check(self.device.lib.rt_cmd_trace_rays(self.device.ctx, C.byref(push), sbt_p, C.byref(d),
                                                            Device.stream_handle(stream)))


class FrameLoop:
    """The reference's double-buffered frame loop (src/main.rs:600-668,
    1131-1170): `frames_in_flight` frames, each with its own instance buffer,
    TLAS clone, uniforms, image and CUDA stream (the Vulkan fences and
    semaphores become stream order).  Frame k uses slot k % frames_in_flight,
    so frame N+1's instance upload, TLAS rebuild and ray generation run while
    frame N is still being traced."""

    def __init__(self, device: Device, gpu_scene: GpuScene, width: int, height: int, frames_in_flight: int = 2,
                 radiance: bool = False):
        self.device = device
        self.gpu_scene = gpu_scene
        self.slots = [PerFrameResources(device, gpu_scene, width, height, radiance=radiance, clone_tlas=True)
                      for _ in range(frames_in_flight)]
        self.streams = [torch.cuda.Stream() for _ in range(frames_in_flight)]
        self.scratch = [ScratchBuffer(f"frame scratch {i}") for i in range(frames_in_flight)]

    def begin(self) -> None:
        """Orders every slot after the work already queued on the current stream."""
        ev = torch.cuda.Event()
        ev.record()
        for s in self.streams:
            s.wait_event(ev)

    def record(self, k: int, max_trace_depth: int, shadow_ray_count: int, instances=None, instances_host=None,
               uniforms_dev=None, image_host=None, flags: int = 0, before=None,
               refit: bool = False, image_direct: bool = False) -> PerFrameResources:
        """Frame k: new instance records (a device tensor, or pinned host bytes
        copied in on the slot's stream), TLAS rebuild (or, with refit, the
        in-place update of DefaultScene::write_resources, scene.rs:167-204),
        uniforms (a device copy), the trace, and optionally the image in
        pinned host memory: copied there after the frame, or with
        image_direct written there by the output kernel itself (through the
        buffer's mapping into the GPU's address space)."""
        i = k % len(self.slots)
        fr, st = self.slots[i], self.streams[i]
        with torch.cuda.stream(st):
            if before is not None:
                before(st)
            if instances_host is not None:
                fr.instances_buffer.copy_(instances_host, non_blocking=True)
                instances = fr.instances_buffer
            if instances is not None and refit:
                fr.tlas.update_tlas(self.device, instances, fr.num_instances, self.scratch[i], st)
            elif instances is not None:
                fr.tlas.rebuild_tlas(self.device, instances, fr.num_instances, self.scratch[i], st)
            if uniforms_dev is not None:
                fr.uniforms_buffer.copy_(uniforms_dev, non_blocking=True)
            direct = image_host is not None and image_direct
            fr.record(max_trace_depth, shadow_ray_count, flags, stream=st,
                      image_address=image_host.data_ptr() if direct else None)
            if image_host is not None and not direct:
                image_host.copy_(fr.image, non_blocking=True)
        return fr

    def end(self) -> None:
        """Makes the current stream wait for every slot."""
        cur = torch.cuda.current_stream()
        for s in self.streams:
            ev = torch.cuda.Event()
            ev.record(s)
            cur.wait_event(ev)


def batch_scene(frame: PerFrameResources, max_trace_depth: int, shadow_ray_count: int,
                flags: int = 0, uniforms_address: int | None = None,
                image_address: int | None = None) -> abi.RtBatchScene:
    """The RtBatchScene of one frame (its scene's own texture table, if any).
    uniforms_address / image_address replace the frame's own uniform buffer
    and image: any device address, or a pinned host pointer, which the output
    kernel then writes over the mapped host path."""
    b = abi.RtBatchScene()
    uni = uniforms_address if uniforms_address is not None else frame.uniforms_buffer.data_ptr()
    b.push = frame.gpu_scene.push_constants(uni, frame.tlas)
    gs = frame.gpu_scene
    if gs.texture_table is not None:
        b.texture_table = gs.texture_table.data_ptr()
        b.texture_count = gs.texture_count
    d = b.desc
    d.width, d.height = frame.width, frame.height
    d.max_trace_depth = max_trace_depth
    d.shadow_ray_count = shadow_ray_count
    d.flags = flags
    d.image_address = image_address if image_address is not None else frame.image.data_ptr()
    d.radiance_address = frame.radiance.data_ptr() if frame.radiance is not None else 0
    return b


def trace_batch(device: Device, scenes: list[abi.RtBatchScene], flags: int = 0,
                sbt: abi.RtShaderBindingTable | None = None, stream=None) -> None:
    """All frames in one rt_cmd_trace_rays_batched call."""
    arr = (abi.RtBatchScene * max(len(scenes), 1))(*scenes)
    sbt_p = C.byref(sbt) if sbt is not None else None
    device.check(device.lib.rt_cmd_trace_rays_batched(device.ctx, arr, len(scenes), sbt_p, flags,
                                                      Device.stream_handle(stream)))


def render(device: Device, scene: Scene, radiance: bool = True, flags: int = 0, gpu_scene: GpuScene | None = None):
    """Builds a scene (unless `gpu_scene` is given), renders one frame and
    returns (image, radiance, stats)."""
    gs = gpu_scene or GpuScene(device, scene)
    fr = PerFrameResources(device, gs, scene.width, scene.height, radiance=radiance)
    fr.write_uniforms(scene.uniforms)
    device.read_stats(reset=True)
    fr.record(scene.max_trace_depth, scene.shadow_ray_count, flags, scene.sbt)
    stats = device.read_stats(reset=True)
    img = fr.image.cpu().numpy()
    rad = fr.radiance.cpu().numpy() if radiance else None
    return img, rad, stats


def trace_ray_buffer(device: Device, gpu_scene: GpuScene, rays: np.ndarray, ray_flags: int = 0,
                     cull_mask: int = 0xFF, sbt_offset: int = 0, with_models: bool = True,
                     sbt: abi.RtShaderBindingTable | None = None):
    """Traversal-only query of `rays` (RAY_DTYPE) against the scene's TLAS."""
    rb = Device.upload(rays)
    hb = Device.alloc(len(rays) * abi.HIT_DTYPE.itemsize)
    push = gpu_scene.push_constants(0) if with_models else abi.RtPushConstantBufferAddresses()
    device.check(device.lib.rt_cmd_trace_ray_buffer(device.ctx, gpu_scene.tlas.device_address(), C.byref(push),
                                                    C.byref(sbt) if sbt is not None else None, ray_flags, cull_mask,
                                                    sbt_offset, rb.data_ptr(), len(rays), hb.data_ptr(),
                                                    Device.stream_handle()))
    torch.cuda.synchronize()
    return hb.cpu().numpy().view(abi.HIT_DTYPE)


def resident_bytes(gpu_scene: GpuScene) -> int:
    """Device bytes a scene keeps resident: BLASes, TLAS, instance and model
    buffers, and its textures."""
    n = gpu_scene.tlas.size + gpu_scene.instances_buffer.numel() + gpu_scene.model_info_buffer.numel()
    for m in gpu_scene.models:
        n += m.blas.size + m.position_buffer.numel() + m.normal_buffer.numel() + m.uv_buffer.numel()
        n += m.geometry_info_buffer.numel() + sum(ib.numel() for ib in m.index_buffers)
    n += sum(t.numel() for t in gpu_scene._texture_refs)
    if gpu_scene.texture_table is not None:
        n += gpu_scene.texture_table.numel()
    return int(n)


class Server:
    """The serving loop of librtcore (rt_server_*): resident scenes, requests
    admitted by an HBM budget and rendered in continuous batches.  The device
    context must be thread-safe (Device(threadsafe=True))."""

    def __init__(self, device: Device, budget_bytes: int, max_batch_requests: int = 32, max_batch_pixels: int = 0,
                 max_in_flight: int = 2, max_batch_shadow_rays: int = 0):
        self.device = device
        cfg = abi.RtServerConfig(int(budget_bytes), max_batch_requests, max_batch_pixels, max_in_flight,
                                 max_batch_shadow_rays)
        self.handle = C.c_void_p()
        device.check(device.lib.rt_server_create(device.ctx, C.byref(cfg), C.byref(self.handle)))
        self.scenes = []

    def add_scene(self, gpu_scene: GpuScene) -> int:
        if gpu_scene.texture_table is None:
            raise ValueError("a served scene needs its own texture table (GpuScene(own_textures=True))")
        s = abi.RtServeScene()
        s.acceleration_structure = gpu_scene.tlas.device_address()
        s.model_info = gpu_scene.model_info_buffer.data_ptr()
        s.texture_table = gpu_scene.texture_table.data_ptr()
        s.texture_count = gpu_scene.texture_count
        s.resident_bytes = resident_bytes(gpu_scene)
        sid = C.c_uint32()
        self.device.check(self.device.lib.rt_server_add_scene(self.handle, C.byref(s), C.byref(sid)))
        self.scenes.append(gpu_scene)
        return sid.value

    def submit(self, scene: int, uniforms: abi.RtUniforms, width: int, height: int, max_trace_depth: int = 2,
               shadow_ray_count: int = 2, image_device: int = 0, image_host: int = 0, flags: int = 0) -> int:
        r = abi.RtServeRequest()
        r.uniforms = uniforms
        r.scene, r.width, r.height = scene, width, height
        r.max_trace_depth, r.shadow_ray_count, r.flags = max_trace_depth, shadow_ray_count, flags
        r.image_device, r.image_host = image_device, image_host
        t = C.c_uint64()
        self.device.check(self.device.lib.rt_server_submit(self.handle, C.byref(r), C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000) -> abi.RtServeResult:
        out = abi.RtServeResult()
        self.device.check(self.device.lib.rt_server_wait(self.handle, ticket, timeout_ms, C.byref(out)))
        return out

    def stats(self) -> dict:
        s = abi.RtServeStats()
        self.device.check(self.device.lib.rt_server_stats(self.handle, C.byref(s)))
        return s.as_dict()

    def close(self) -> None:
        if self.handle:
            self.device.check(self.device.lib.rt_server_destroy(self.handle))
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
