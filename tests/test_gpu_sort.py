"""The BVH builder's key sort (rt_debug_sort_pairs runs it on its own).

Every BLAS and TLAS build sorts its primitives' 30-bit Morton codes with
their indices as values; the order must be the stable one, because the
hierarchy is built over it.  Above one sort tile (2048 keys) the sort is
the onesweep scheme (per-digit passes with decoupled look-back across
partitions of 3840 keys); these sizes cover one block, the tile edges, a
ragged last partition, duplicate-heavy and full 32-bit keys, and the
precision mesh's 10,485,760 keys.  The reference is numpy's stable argsort.
"""
import ctypes as C

import numpy as np
import pytest

from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu


def _sort_on_device(device, keys, vals):
    import torch

    n = len(keys)
    need = C.c_uint64()
    device.check(device.lib.rt_debug_sort_pairs(0, 0, n, 0, 0, C.byref(need), None))
    k = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    v = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    scratch = torch.empty(int(need.value), dtype=torch.uint8, device="cuda")
    device.check(device.lib.rt_debug_sort_pairs(k.data_ptr(), v.data_ptr(), n, scratch.data_ptr(), need.value,
                                                None, None))
    return k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def _check(device, keys):
    vals = np.arange(len(keys), dtype=np.uint32)[::-1].copy()  # values unrelated to the keys' order
    gk, gv = _sort_on_device(device, keys, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(gk, keys[order])
    assert np.array_equal(gv, vals[order]), "not the stable order"


@pytest.mark.parametrize("n", [1, 2, 1000, 2048, 2049, 3840, 3841, 7681, 100_003])
@pytest.mark.parametrize("kind", ["morton", "duplicates", "full32"])
def test_sort_matches_stable_argsort(device, n, kind):
    rng = scenes.Pcg32(n + 17, 0x50)
    raw = rng.u32_array(n).astype(np.uint32)
    if kind == "morton":
        keys = raw & np.uint32((1 << 30) - 1)
    elif kind == "duplicates":
        keys = (raw % np.uint32(7)) << np.uint32(8) | (raw & np.uint32(3)) << np.uint32(24)
    else:
        keys = raw
    _check(device, keys.astype(np.uint32))


def test_sort_of_precision_mesh_morton_codes(device):
    """10,485,760 keys shaped like the precision mesh's Morton codes: sorted
    runs broken up (a surface's codes are far from uniform)."""
    n = 10_485_760
    rng = scenes.Pcg32(9, 0x50)
    coarse = (rng.u32_array(n).astype(np.uint64) % np.uint64(4096)).astype(np.uint32) << np.uint32(18)
    fine = rng.u32_array(n).astype(np.uint32) & np.uint32((1 << 18) - 1)
    _check(device, coarse | fine)


def test_sort_rejects_small_scratch(device):
    need = C.c_uint64()
    device.check(device.lib.rt_debug_sort_pairs(0, 0, 100_000, 0, 0, C.byref(need), None))
    r = device.lib.rt_debug_sort_pairs(256, 256, 100_000, 256, need.value - 1, None, None)
    assert r == abi.RT_ERR_INVALID
