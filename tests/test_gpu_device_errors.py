"""Device-side error statuses of the traversal, made to happen on purpose.

The traversal bounds every loop that follows a structure and range-checks
every reference it reads (RT_ERR_TIMEOUT after 2^22 steps of one ray,
RT_ERR_STACK_OVERFLOW when a push would pass the 64-entry stack, RT_ERR_BAD_AS
for a node or leaf reference outside the structure's counts).  These tests
write BLAS node arrays by hand into a real build's memory, every reference in
range except where the range check is the point, and check that the status
is reported in the context statistics and that a following valid launch runs
clean:

* a node whose only child is itself: the ray steps until the bound;
* a chain of 12 nodes, each with its next node as the nearest child and
  seven leaves behind it: 7 pushes per level overflow the stack;
* a child reference past the node count and a leaf past the triangle count:
  skipped and reported.
"""
import numpy as np
import pytest

from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu

HEADER_BYTES, NODE_BYTES = 512, 256
LEAF, EMPTY = 0x80000000, 0xFFFFFFFF
ERR_BIT = {abi.RT_ERR_STACK_OVERFLOW: 1 << abi.RT_ERR_STACK_OVERFLOW, abi.RT_ERR_TIMEOUT: 1 << abi.RT_ERR_TIMEOUT,
           abi.RT_ERR_BAD_AS: 1 << abi.RT_ERR_BAD_AS}


def _host():
    from rtgallery import host

    return host


def _torus_scene():
    pos, nrm, uv, idx = scenes.torus(1.0, 0.35, 16, 8)
    m = scenes.Model(pos, nrm, uv, [scenes.Geometry(idx, True)], "torus16x8")
    inst = scenes.instance_records(scenes.affine(np.eye(3), [0, 0, 0])[None], np.array([0]), np.array([0]), 0)
    return scenes.Scene([m], {}, inst, scenes.scene_small(8, 8).uniforms, 8, 8, name="torus")


class Blob:
    """A BLAS blob on the host: header fields and the FP32 wide-node array."""

    def __init__(self, blas):
        self.blas = blas
        self.bytes = blas.buffer.cpu().numpy().copy()
        h = self.bytes[:HEADER_BYTES].view(np.uint32)
        self.node_count, self.prim_count = int(h[4]), int(h[5])
        # header: 8 x u32 (magic .. node_bytes), u64 total_size @32, nodes_offset @40, prims_offset @48,
        # parents_offset @56, float bounds_lo[3] @64, bounds_hi[3] @76
        self.nodes_offset = int(self.bytes[:HEADER_BYTES].view(np.uint64)[5])
        f = self.bytes[:HEADER_BYTES].view(np.float32)
        self.lo, self.hi = f[16:19].copy(), f[19:22].copy()

    def node(self, i):
        o = self.nodes_offset + i * NODE_BYTES
        return self.bytes[o:o + NODE_BYTES]

    def write_node(self, i, boxes, refs):
        """boxes: 8 x (lo3, hi3) or None (empty); refs: 8 child references."""
        n = self.node(i)
        f = n[:192].view(np.float32).reshape(6, 8)  # lox hix loy hiy loz hiz
        for k in range(8):
            if boxes[k] is None:
                lo, hi = (1.0, 1.0, 1.0), (-1.0, -1.0, -1.0)
            else:
                lo, hi = boxes[k]
            f[0, k], f[1, k], f[2, k], f[3, k], f[4, k], f[5, k] = lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]
        n[192:224].view(np.uint32)[:] = np.array(refs, np.uint32)

    def upload(self):
        import torch

        self.blas.buffer.copy_(torch.from_numpy(self.bytes))


def _rays_along_x(count, spread=0.02):
    rays = np.zeros(count, abi.RAY_DTYPE)
    t = np.linspace(-spread, spread, count, dtype=np.float32)
    rays["origin"] = np.stack([np.full(count, -10.0, np.float32), t, t * 0.5], 1)
    rays["direction"] = np.array([1.0, 0.0, 0.0], np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = 1e4
    return rays


def _trace_status(device, gs, rays):
    device.read_stats(reset=True)
    hits = _host().trace_ray_buffer(device, gs, rays, with_models=False)
    return hits, device.read_stats(reset=True)["status"]


def _clean_launch_after(device):
    """A valid scene traced after the faulty one: no status, hits as usual."""
    sc = scenes.scene_small(32, 32)
    gs = _host().GpuScene(device, sc)
    hits, status = _trace_status(device, gs, scenes.random_rays(4096, 3, 12.0))
    assert status == 0
    assert (hits["instance_id"] != 0xFFFFFFFF).sum() > 100


@pytest.fixture
def torus(device):
    gs = _host().GpuScene(device, _torus_scene())
    blob = Blob(gs.models[0].blas)
    assert blob.node_count >= 13 and blob.prim_count == 256
    return gs, blob


def test_self_referencing_node_times_out(device, torus):
    gs, blob = torus
    whole = (blob.lo, blob.hi)
    blob.write_node(0, [whole] + [None] * 7, [0] + [EMPTY] * 7)  # the root's only child is the root
    blob.upload()
    hits, status = _trace_status(device, gs, _rays_along_x(64))
    assert status & ERR_BIT[abi.RT_ERR_TIMEOUT]
    assert not status & ERR_BIT[abi.RT_ERR_BAD_AS]
    _clean_launch_after(device)


def test_deep_chain_overflows_the_stack(device, torus):
    gs, blob = torus
    whole = (blob.lo, blob.hi)
    mid = (blob.lo + blob.hi) * 0.5
    behind = ((mid[0], blob.lo[1], blob.lo[2]), blob.hi)  # entered later by a ray along +x
    for i in range(12):
        nxt = i + 1 if i < 11 else None
        boxes = [whole if nxt is not None else behind] + [behind] * 7
        refs = [nxt if nxt is not None else LEAF] + [LEAF] * 7  # leaves: triangle 0
        blob.write_node(i, boxes, refs)
    blob.upload()
    hits, status = _trace_status(device, gs, _rays_along_x(32))
    assert status & ERR_BIT[abi.RT_ERR_STACK_OVERFLOW]
    assert not status & (ERR_BIT[abi.RT_ERR_TIMEOUT] | ERR_BIT[abi.RT_ERR_BAD_AS])
    _clean_launch_after(device)


def test_out_of_range_references_are_skipped_and_reported(device, torus):
    gs, blob = torus
    whole = (blob.lo, blob.hi)
    past_nodes = blob.node_count + 5
    past_tris = LEAF | (1 << 28) | (blob.prim_count - 1)  # 2 triangles from the last one
    blob.write_node(0, [whole, whole] + [None] * 6, [past_nodes, past_tris] + [EMPTY] * 6)
    blob.upload()
    hits, status = _trace_status(device, gs, _rays_along_x(32))
    assert status & ERR_BIT[abi.RT_ERR_BAD_AS]
    assert (hits["instance_id"] == 0xFFFFFFFF).all()  # nothing valid was left to hit
    _clean_launch_after(device)
