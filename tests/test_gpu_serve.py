"""The serving loop (rt_server_*): resident scenes, budget admission,
continuous batching.

A request's image must be byte-identical whether it is rendered alone (a
server that batches one request at a time) or inside a mix of other
requests, and one request is also checked against the oracle.  The HBM
budget bounds the server's bytes: requests that do not fit wait, requests
that can never fit are refused.
"""
import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu

RES = [(64, 48), (96, 64), (33, 17), (128, 96), (80, 80)]


def _host():
    from rtgallery import host

    return host


@pytest.fixture(scope="module")
def served():
    host = _host()
    dev = host.Device(threadsafe=True)
    specs = [scenes.scene_small(64, 64), scenes.scene_gallery(96, 64), scenes.scene_full(2, 96, 54)]
    gscenes = [host.GpuScene(dev, sc, own_textures=True) for sc in specs]
    yield dev, specs, gscenes
    dev.close()


def _requests(n, seed):
    rng = scenes.Pcg32(seed, 0x5E)
    out = []
    for i in range(n):
        w, h = RES[int(rng.next_u32() % len(RES))]
        u = scenes.random_view_uniforms(rng, w, h, frame=i)
        out.append(dict(scene=i % 3, uniforms=u, width=w, height=h, max_trace_depth=1 + int(rng.next_u32() % 3),
                        shadow_ray_count=1 + int(rng.next_u32() % 8)))
    return out


def _serve(dev, gscenes, reqs, budget, max_batch, in_flight):
    import torch

    host = _host()
    srv = host.Server(dev, budget, max_batch_requests=max_batch, max_in_flight=in_flight)
    ids = [srv.add_scene(g) for g in gscenes]
    imgs = [torch.zeros(r["height"] * r["width"] * 4, dtype=torch.uint8, device="cuda") for r in reqs]
    torch.cuda.synchronize()
    tickets = [srv.submit(ids[r["scene"]], r["uniforms"], r["width"], r["height"], r["max_trace_depth"],
                          r["shadow_ray_count"], image_device=img.data_ptr()) for r, img in zip(reqs, imgs)]
    results = [srv.wait(t, 120000) for t in tickets]
    stats = srv.stats()
    srv.close()
    torch.cuda.synchronize()
    return imgs, results, stats


def test_request_identical_alone_and_in_mix(served):
    import torch

    dev, specs, gscenes = served
    reqs = _requests(24, 3)
    alone, res_a, _ = _serve(dev, gscenes, reqs, 8 << 30, 1, 1)
    mix, res_m, st = _serve(dev, gscenes, reqs, 8 << 30, 16, 2)
    assert all(r.state == abi.RT_SERVE_DONE and r.status == 0 for r in res_a + res_m)
    assert all(r.batch_requests == 1 for r in res_a)
    assert max(r.batch_requests for r in res_m) > 1, "the mix never batched"
    for k in range(len(reqs)):
        assert torch.equal(alone[k], mix[k]), f"request {k} differs alone vs in the mix"
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    # one request against the oracle
    k = 5
    r = reqs[k]
    o_img, _, _ = O.OracleScene(specs[r["scene"]]).render(uniforms=r["uniforms"], width=r["width"],
                                                            height=r["height"], max_trace_depth=r["max_trace_depth"],
                                                            shadow_ray_count=r["shadow_ray_count"])
    img = mix[k].cpu().numpy().reshape(r["height"], r["width"], 4)
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1


def test_budget_admission(served):
    host = _host()
    dev, specs, gscenes = served
    resident = sum(host.resident_bytes(g) for g in gscenes)
    reqs = _requests(30, 9)
    budget = resident + (48 << 20)  # room for a few frames and one batch workspace at a time
    _, res, st = _serve(dev, gscenes, reqs, budget, 16, 2)
    assert all(r.state == abi.RT_SERVE_DONE and r.status == 0 for r in res)
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["peak_bytes"] <= budget
    # a request that cannot fit even alone is refused at submit
    srv = host.Server(dev, budget, max_batch_requests=16)
    sid = [srv.add_scene(g) for g in gscenes][0]
    with pytest.raises(abi.RtError) as e:
        srv.submit(sid, reqs[0]["uniforms"], 8192, 8192, 2, 8)
    assert e.value.status == abi.RT_ERR_TOO_LARGE
    srv.close()
    # and a scene that does not fit the budget is refused
    small = host.Server(dev, 1 << 20)
    with pytest.raises(abi.RtError) as e:
        small.add_scene(gscenes[2])
    assert e.value.status == abi.RT_ERR_OOM
    small.close()


def test_server_needs_threadsafe_context(device):
    host = _host()
    with pytest.raises(abi.RtError):
        host.Server(device, 1 << 30)


def _serve_limited(dev, gscenes, reqs, budget, max_batch, in_flight, max_pixels, max_shadow, host_images=False):
    """Like _serve, with batch limits (the server then reserves its workspace
    at creation); host_images: the images go to page-locked host buffers,
    which the output kernel writes directly."""
    import torch

    host = _host()
    srv = host.Server(dev, budget, max_batch_requests=max_batch, max_in_flight=in_flight,
                      max_batch_pixels=max_pixels, max_batch_shadow_rays=max_shadow)
    after_create = srv.stats()
    ids = [srv.add_scene(g) for g in gscenes]
    if host_images:
        imgs = [torch.zeros(r["height"] * r["width"] * 4, dtype=torch.uint8).pin_memory() for r in reqs]
        kw = [dict(image_host=img.data_ptr()) for img in imgs]
    else:
        imgs = [torch.zeros(r["height"] * r["width"] * 4, dtype=torch.uint8, device="cuda") for r in reqs]
        kw = [dict(image_device=img.data_ptr()) for img in imgs]
    torch.cuda.synchronize()
    tickets = [srv.submit(ids[r["scene"]], r["uniforms"], r["width"], r["height"], r["max_trace_depth"],
                          r["shadow_ray_count"], **k) for r, k in zip(reqs, kw)]
    results = [srv.wait(t, 120000) for t in tickets]
    stats = srv.stats()
    srv.close()
    torch.cuda.synchronize()
    return [i.cpu() for i in imgs], results, stats, after_create


def _slots(r):
    return ((r["width"] + 7) // 8 * 8) * ((r["height"] + 3) // 4 * 4)


def test_full_hd_request_in_a_mix_with_batch_limits(served):
    """A 1920x1080 request with 8 shadow rays among small ones, through a
    server with batch limits (ray slots and shadow rays) and a reserved
    workspace: every image equals the request rendered alone, no batch
    exceeds the limits unless it holds one request, the reserved workspace
    is counted from creation on, and the 1080p request matches the oracle."""
    dev, specs, gscenes = served
    reqs = _requests(24, 11)
    big = dict(scene=1, uniforms=scenes.random_view_uniforms(scenes.Pcg32(77, 1), 1920, 1080, frame=3),
               width=1920, height=1080, max_trace_depth=3, shadow_ray_count=8)
    reqs.insert(7, big)
    limit_px, limit_sh = 1 << 20, 4 << 20
    alone, res_a, _ = _serve(dev, gscenes, reqs, 16 << 30, 1, 1)
    mix, res_m, st, created = _serve_limited(dev, gscenes, reqs, 16 << 30, 16, 2, limit_px, limit_sh)
    assert all(r.state == abi.RT_SERVE_DONE and r.status == 0 for r in res_a + res_m)
    assert created["peak_bytes"] > (64 << 20), "the reserved workspace is not counted at creation"
    for k in range(len(reqs)):
        assert np.array_equal(alone[k].cpu().numpy(), mix[k].numpy()), f"request {k} differs alone vs in the mix"
    by_batch = {}
    for r, q in zip(res_m, reqs):
        by_batch.setdefault(r.batch, []).append(q)
    assert max(len(v) for v in by_batch.values()) > 1, "the mix never batched"
    for b, qs in by_batch.items():
        if len(qs) > 1:
            assert sum(_slots(q) for q in qs) <= limit_px, b
            assert sum(q["width"] * q["height"] * q["shadow_ray_count"] for q in qs) <= limit_sh, b
    assert res_m[7].batch_requests == 1  # beyond both limits on its own: rendered alone
    o_img, _, _ = O.OracleScene(specs[1]).render(uniforms=big["uniforms"], width=1920, height=1080,
                                                 max_trace_depth=3, shadow_ray_count=8)
    img = mix[7].numpy().reshape(1080, 1920, 4)
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1


def test_page_locked_host_images_are_written_directly(served):
    """Requests whose image_host is page-locked get their image from the
    output kernel itself (no server frame buffer): the same bytes as device
    images."""
    dev, specs, gscenes = served
    reqs = _requests(16, 21)
    dev_imgs, _, _, _ = _serve_limited(dev, gscenes, reqs, 8 << 30, 8, 2, 1 << 20, 8 << 20)
    host_imgs, res, st, _ = _serve_limited(dev, gscenes, reqs, 8 << 30, 8, 2, 1 << 20, 8 << 20, host_images=True)
    assert all(r.state == abi.RT_SERVE_DONE and r.status == 0 for r in res)
    for k in range(len(reqs)):
        assert np.array_equal(dev_imgs[k].numpy(), host_imgs[k].numpy()), k
