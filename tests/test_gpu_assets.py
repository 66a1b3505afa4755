"""The reference's default scene, built from asset files decoded by
librtcore.so (GLB models, PNG textures), rendered on the GPU and checked
against the CPU oracle on the same decoded arrays.

The asset files are the package's synthetic stand-ins (same kinds and sizes
as the reference's: a 45,448-triangle figure with a linearly filtered 512^2
texture, an alpha-masked fence, 16-bit blue noise ...).  The frame loop is
the reference's: the figure turns by 0.05 rad per frame and the TLAS is
refitted in place (scene.rs:163-204), two frames in flight.
"""
import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import assets

pytestmark = pytest.mark.gpu
RADIANCE_TOL = 1e-3


@pytest.fixture(scope="module")
def files():
    return assets.standin_assets()


def test_default_scene_render_matches_oracle(device, files):
    from rtgallery import host

    sc = assets.default_scene(files, 256, 144)
    img, rad, st = host.render(device, sc, radiance=True)
    o_img, o_rad, o_st = O.OracleScene(sc).render()
    for k in ("traversals", "primary_rays", "secondary_rays", "shadow_rays"):
        assert st[k] == o_st[k], (k, st[k], o_st[k])
    assert st["status"] == 0
    assert np.abs(rad - o_rad).max() <= RADIANCE_TOL
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1
    assert st["secondary_rays"] > 0 and st["shadow_rays"] > 0
    # the figure's texture is sampled: its pixels are not one flat colour
    assert len(np.unique(img.reshape(-1, 4), axis=0)) > 1000


def test_default_scene_frame_loop_refit_matches_oracle(device, files):
    """Four frames of the reference's loop: new figure transform, in-place TLAS
    refit on that frame's slot, trace; every frame equals the oracle."""
    import torch

    from rtgallery import host

    W, H, N = 192, 108, 4
    sc0 = assets.default_scene(files, W, H, frame=0)
    gs = host.GpuScene(device, sc0)
    insts = [assets.default_scene_instances(0, k) for k in range(N)]
    unis = [assets.default_scene_uniforms(W, H, k + 1) for k in range(N)]
    inst_dev = [host.Device.upload(gs.patch_instances(i)) for i in insts]
    uni_dev = [host.Device.upload(np.frombuffer(bytes(u), np.uint8)) for u in unis]
    loop = host.FrameLoop(device, gs, W, H, frames_in_flight=2, radiance=True)
    imgs = [torch.empty((H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(N)]
    loop.begin()
    for k in range(N):
        loop.record(k, sc0.max_trace_depth, sc0.shadow_ray_count, instances=inst_dev[k], uniforms_dev=uni_dev[k],
                    image_host=imgs[k], refit=True)
    loop.end()
    torch.cuda.synchronize()
    o = O.OracleScene(sc0)
    for k in range(N):
        o.set_instances(insts[k])
        o_img, _, _ = o.render(uniforms=unis[k])
        diff = np.abs(imgs[k].numpy().astype(int) - o_img.astype(int)).max()
        assert diff <= 1, f"frame {k}: {diff}"
    for fr in loop.slots:
        assert fr.tlas.info(device).status == 0
    assert not np.array_equal(imgs[0].numpy(), imgs[N - 1].numpy())
