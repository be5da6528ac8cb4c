"""The fused multi-view render (ubs.render) against the drop-in operator
sequence of the reference model's render (ubs.scene.render_view, which calls
the gsplat-compatible operators one by one) on the same scenes.

Both paths evaluate the same mathematics with different kernel fusion and
summation order, so images agree to FP32 rounding (1e-5 max abs) and
gradients to 1e-4 relative (L2 per parameter tensor)."""
import math

import numpy as np
import pytest
import torch

from ubs import scene as S
from ubs.render import Renderer, Views

pytestmark = pytest.mark.gpu
DEV = "cuda"


def rel_l2(a, b):
    a, b = a.detach().double(), b.detach().double()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


def make_params(N, D, seed, xyz_range=1.0):
    p = S.synthetic_params(N, D, seed=seed, xyz_range=xyz_range, device=DEV)
    # larger spatial scales than the benchmark so small images get dense coverage
    p["scale"][:, :3] += 1.5
    return p


def dropin_render(p, cam, bg, exact=False):
    from gsplat.cuda import _wrapper as Wr
    ri, rj = S.rest_indices(p["scale"].shape[1], DEV)
    leaves = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    prev = Wr.get_cond_grad_mode()
    Wr.set_cond_grad_mode("exact" if exact else "reference")
    try:
        img, alphas, _ = S.render_view(leaves, cam, bg, ri, rj)
    finally:
        Wr.set_cond_grad_mode(prev)
    return img.permute(1, 2, 0), alphas[0, ..., 0], leaves


def fused_render(p, cams, bg, exact=False, capacity=None):
    r = Renderer(dim=p["scale"].shape[1], capacity=capacity, exact_cond_grad=exact)
    views = Views(cams, device=DEV)
    leaves = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    colors, alphas = r.render(leaves, views, bg)
    return r, views, colors, alphas, leaves


@pytest.mark.parametrize("D,exact", [(6, False), (6, True), (7, False)])
def test_fused_single_view_matches_dropin(D, exact):
    p = make_params(6000, D, seed=D)
    cam = S.orbit_view(5, 3.0, 320, 240, 280.0, 280.0, timestamp=0.37, device=DEV)
    bg = torch.tensor([0.1, 0.2, 0.3], device=DEV)
    img_d, alpha_d, leaves_d = dropin_render(p, cam, bg, exact)
    _, views, colors, alphas, leaves_f = fused_render(p, [cam], bg, exact)
    img_f = views.split(colors)[0]
    assert float((img_f - img_d).detach().abs().max()) < 1e-5
    assert float((alphas.view(240, 320) - alpha_d).abs().max()) < 1e-5
    assert float(alpha_d.mean()) > 0.05  # the scene covers the image
    g = torch.Generator().manual_seed(3)
    w = torch.randn(240, 320, 3, generator=g).to(DEV)
    wa = torch.randn(240, 320, generator=g).to(DEV)
    ((img_d * w).sum() + (alpha_d * wa).sum()).backward()
    ((img_f * w).sum() + (alphas.view(240, 320) * wa).sum()).backward()
    for k in leaves_d:
        assert rel_l2(leaves_f[k].grad, leaves_d[k].grad) < 1e-4, (k, rel_l2(leaves_f[k].grad,
                                                                         leaves_d[k].grad))


def test_fused_multiview_mixed_resolution():
    p = make_params(5000, 6, seed=11)
    cams = [S.orbit_view(1, 3.0, 160, 120, 150.0, 150.0, device=DEV),
            S.orbit_view(2, 3.5, 200, 96, 170.0, 170.0, device=DEV),
            S.orbit_view(3, 2.8, 96, 96, 90.0, 90.0, device=DEV)]
    bgs = torch.rand(3, 3, generator=torch.Generator().manual_seed(0)).to(DEV)
    _, views, colors, alphas, leaves_f = fused_render(p, cams, bgs)
    imgs = views.split(colors)
    g = torch.Generator().manual_seed(5)
    ws = [torch.randn(c.height, c.width, 3, generator=g).to(DEV) for c in cams]
    total_f = sum((im * w).sum() for im, w in zip(imgs, ws))
    total_f.backward()
    grads = {k: torch.zeros_like(v) for k, v in p.items()}
    for v, cam in enumerate(cams):
        img_d, _, leaves_d = dropin_render(p, cam, bgs[v])
        assert float((imgs[v] - img_d).abs().max()) < 1e-5, v
        (img_d * ws[v]).sum().backward()
        for k in grads:
            grads[k] += leaves_d[k].grad
    for k in grads:
        assert rel_l2(leaves_f[k].grad, grads[k]) < 1e-4, (k, rel_l2(leaves_f[k].grad, grads[k]))


@pytest.mark.parametrize("N,D", [(50, 7), (129, 6)])
def test_fused_multiview_few_primitives(N, D):
    # the per-primitive kernels work in CTAs of 128 (view, primitive)
    # entries: with N < 128 one CTA holds entries of three or more views
    p = make_params(N, D, seed=N)
    p["scale"][:, :3] += 1.0
    cams = [S.orbit_view(v, 3.0, 64 + 16 * v, 48, 60.0, 60.0, timestamp=0.1 * v, device=DEV)
            for v in range(4)]
    bgs = torch.rand(4, 3, generator=torch.Generator().manual_seed(1)).to(DEV)
    _, views, colors, alphas, leaves_f = fused_render(p, cams, bgs)
    imgs = views.split(colors)
    g = torch.Generator().manual_seed(9)
    ws = [torch.randn(c.height, c.width, 3, generator=g).to(DEV) for c in cams]
    sum((im * w).sum() for im, w in zip(imgs, ws)).backward()
    grads = {k: torch.zeros_like(v) for k, v in p.items()}
    for v, cam in enumerate(cams):
        img_d, _, leaves_d = dropin_render(p, cam, bgs[v])
        assert float((imgs[v] - img_d).abs().max()) < 1e-5, v
        (img_d * ws[v]).sum().backward()
        for k in grads:
            grads[k] += leaves_d[k].grad
    for k in grads:
        assert rel_l2(leaves_f[k].grad, grads[k]) < 1e-4, (k, rel_l2(leaves_f[k].grad, grads[k]))


def test_fused_many_tiles_match_dropin():
    # 3 views of 1920x1080 at 16x16 tiles: 24,480 (view, tile) buckets, so
    # the single-CTA launch-order pass walks its buckets in many strides
    p = make_params(3000, 6, seed=31)
    cams = [S.orbit_view(40 + v, 3.0, 1920, 1080, 1500.0, 1500.0, device=DEV) for v in range(3)]
    bgs = torch.rand(3, 3, generator=torch.Generator().manual_seed(2)).to(DEV)
    _, views, colors, alphas, _ = fused_render(p, cams, bgs)
    assert views.n_buckets > 16384
    imgs = views.split(colors)
    for v, cam in enumerate(cams):
        img_d, _, _ = dropin_render(p, cam, bgs[v])
        assert float((imgs[v] - img_d).detach().abs().max()) < 1e-5, v
    assert float(alphas.max()) > 0.5


def test_fused_more_buckets_than_one_scan_cta():
    # 9 views of 1920x1080 at 16x16 tiles: 73,440 (view, tile) buckets, more
    # than the one-CTA scan takes, so the replicated bucket counters are
    # folded, scanned device-wide and turned into replica cursors by separate
    # kernels and the launch order comes from the order kernel
    p = make_params(3000, 6, seed=37)
    cams = [S.orbit_view(60 + v, 3.0, 1920, 1080, 1500.0, 1500.0, device=DEV) for v in range(9)]
    bgs = torch.rand(9, 3, generator=torch.Generator().manual_seed(4)).to(DEV)
    _, views, colors, alphas, leaves = fused_render(p, cams, bgs)
    assert views.n_buckets > 65536
    imgs = views.split(colors)
    g = torch.Generator().manual_seed(5)
    wts = [torch.rand(imgs[v].shape, generator=g).to(DEV) for v in range(9)]
    sum((imgs[v] * wts[v]).sum() for v in range(9)).backward()
    grads = {k: torch.zeros_like(v) for k, v in p.items()}
    for v, cam in enumerate(cams):
        img_d, _, leaves_d = dropin_render(p, cam, bgs[v])
        assert float((imgs[v] - img_d).detach().abs().max()) < 1e-5, v
        (img_d * wts[v]).sum().backward()
        for k in grads:
            grads[k] += leaves_d[k].grad
    for k in grads:
        assert rel_l2(leaves[k].grad, grads[k]) < 1e-4, (k, rel_l2(leaves[k].grad, grads[k]))
    assert float(alphas.max()) > 0.5


def test_fused_capacity_overflow_is_recovered():
    p = make_params(4000, 6, seed=21)
    cam = S.orbit_view(7, 3.0, 256, 192, 220.0, 220.0, device=DEV)
    bg = torch.zeros(3, device=DEV)
    r, views, colors, _, _ = fused_render(p, [cam], bg, capacity=1000)
    assert r.last_isects > 1000 and r.capacity > r.last_isects
    img_d, _, _ = dropin_render(p, cam, bg)
    assert float((views.split(colors)[0] - img_d).abs().max()) < 1e-5


def test_fused_unchecked_overflow_is_reported():
    p = make_params(3000, 6, seed=22)
    cam = S.orbit_view(8, 3.0, 200, 150, 180.0, 180.0, device=DEV)
    r = Renderer(dim=6, capacity=500)
    views = Views([cam], device=DEV)
    with torch.no_grad():
        r.render(p, views, check=False)
        with pytest.raises(RuntimeError, match="capacity"):
            r.render(p, views, check=False)
    assert r.capacity > 500
    with torch.no_grad():
        colors, _ = r.render(p, views, check=True)
    img_d, _, _ = dropin_render(p, cam, torch.zeros(3, device=DEV))
    assert float((views.split(colors)[0] - img_d).abs().max()) < 1e-5


def test_graphed_step_matches_eager_and_follows_parameter_updates():
    from ubs.render import GraphedStep
    p = make_params(6000, 6, seed=31)
    cam = S.orbit_view(9, 3.0, 320, 240, 280.0, 280.0, device=DEV)
    g = torch.Generator().manual_seed(8)
    target = torch.rand(240 * 320, 3, generator=g).to(DEV)
    leaves = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    views = Views([cam], device=DEV)
    loss_fn = lambda colors, alphas: (colors - target).abs().mean()  # noqa: E731
    gs = GraphedStep(Renderer(dim=6), leaves, views, None, loss_fn)
    assert gs.launches_per_replay >= 8

    def eager():
        ref = {k: v.detach().clone().requires_grad_(True) for k, v in leaves.items()}
        colors, alphas = Renderer(dim=6).render(ref, Views([cam], device=DEV))
        loss = loss_fn(colors, alphas)
        loss.backward()
        return float(loss), {k: v.grad for k, v in ref.items()}

    for step in range(3):
        loss = float(gs.replay())
        gs.check()
        l_ref, g_ref = eager()
        assert abs(loss - l_ref) <= 1e-6 * abs(l_ref)
        for k in g_ref:
            assert rel_l2(leaves[k].grad, g_ref[k]) < 1e-5, (step, k)
        with torch.no_grad():  # an in-place parameter update, as an optimizer makes
            for v in leaves.values():
                v.add_(0.01 * torch.randn_like(v))


def test_kernel_timer_eager_and_graph_replays():
    from ubs import _lib as L
    from ubs.render import GraphedStep
    p = make_params(3000, 6, seed=41)
    cam = S.orbit_view(4, 3.0, 160, 120, 140.0, 140.0, device=DEV)
    views = Views([cam], device=DEV)
    leaves = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    L.profile_start(256)
    colors, alphas = Renderer(dim=6).render(leaves, views)
    (colors.sum() + alphas.sum()).backward()
    k = L.profile_stop()
    for name in ("scene_prim_fwd", "scene_emit", "bucket_sort_warp", "bucket_scan_order", "raster_fwd",
                 "raster_bwd", "scene_prim_bwd"):
        assert name in k and k[name][0] >= 1 and k[name][1] > 0, (name, k.get(name))
    # fresh leaves: these went through an eager backward on the default stream
    leaves_g = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    gs = GraphedStep(Renderer(dim=6), leaves_g, views, None,
                     lambda c, a: c.square().mean(), before_capture=lambda: L.profile_start(256))
    for _ in range(3):
        gs.replay()
        L.profile_sample()
    k = L.profile_stop()
    assert k["raster_bwd"][0] == 3 and k["raster_fwd"][0] == 3 and k["raster_bwd"][1] > 0


@pytest.mark.parametrize("ts", [8, 24, 32])
def test_fused_tile_sizes_match_dropin(ts):
    from gsplat.cuda import _wrapper as Wr
    p = make_params(4000, 6, seed=50 + ts)
    cam = S.orbit_view(6, 3.0, 250, 170, 220.0, 220.0, device=DEV)
    bg = torch.tensor([0.3, 0.2, 0.1], device=DEV)
    ri, rj = S.rest_indices(6, DEV)
    leaves_d = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    img_d, _, _ = S.render_view(leaves_d, cam, bg, ri, rj, tile_size=ts)
    img_d = img_d.permute(1, 2, 0)
    r = Renderer(dim=6, tile_size=ts)
    views = Views([cam], tile_size=ts, device=DEV)
    leaves_f = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    colors, _ = r.render(leaves_f, views, bg)
    img_f = views.split(colors)[0]
    assert float((img_f - img_d).detach().abs().max()) < 1e-5
    w = torch.randn(170, 250, 3, generator=torch.Generator().manual_seed(1)).to(DEV)
    (img_d * w).sum().backward()
    (img_f * w).sum().backward()
    for k in leaves_d:
        assert rel_l2(leaves_f[k].grad, leaves_d[k].grad) < 1e-4, k


def test_fused_empty_scene_and_nothing_visible():
    """No primitives, or none in front of the camera: the image is the
    background, alphas are zero, gradients are zero, nothing overflows."""
    bg = torch.tensor([0.25, 0.5, 0.75], device=DEV)
    cam = S.orbit_view(1, 3.0, 64, 48, 60.0, 60.0, device=DEV)
    empty = {k: v[:0] for k, v in make_params(10, 6, seed=1).items()}
    r, views, colors, alphas, leaves = fused_render(empty, [cam], bg)
    assert torch.equal(colors, bg.expand_as(colors)) and not alphas.any()
    colors.sum().backward()  # empty gradients, no launch failure
    p = make_params(2000, 6, seed=2)
    with torch.no_grad():
        center = cam.center.to(DEV)
        fwd = torch.inverse(cam.viewmat.to(DEV))[:3, 2]
        p["xyz"].copy_(center - 5.0 * fwd + 0.1 * torch.randn_like(p["xyz"]))  # behind it
    r, views, colors, alphas, leaves = fused_render(p, [cam], bg)
    assert torch.equal(colors, bg.expand_as(colors)) and not alphas.any()
    (colors * torch.rand_like(colors)).sum().backward()
    for k, v in leaves.items():
        assert v.grad is not None and not v.grad.any(), k


@pytest.mark.parametrize("W,H", [(17, 13), (1, 1), (33, 5)])
def test_fused_odd_and_tiny_images_match_dropin(W, H):
    """Partial tiles and single pixels: the fused path agrees with the
    drop-in sequence image for image and gradient for gradient."""
    p = make_params(3000, 6, seed=W + H)
    cam = S.orbit_view(3, 3.0, W, H, 20.0 * max(W, H) / 17, 20.0 * max(W, H) / 17, device=DEV)
    bg = torch.tensor([0.1, 0.2, 0.3], device=DEV)
    img_d, alpha_d, leaves_d = dropin_render(p, cam, bg)
    _, views, colors, alphas, leaves_f = fused_render(p, [cam], bg)
    img_f = views.split(colors)[0]
    assert img_f.shape == (H, W, 3)
    assert float((img_f - img_d).detach().abs().max()) < 1e-5
    g = torch.Generator().manual_seed(1)
    w = torch.randn(H, W, 3, generator=g).to(DEV)
    (img_d * w).sum().backward()
    (img_f * w).sum().backward()
    for k in leaves_d:
        if leaves_d[k].grad.abs().max() > 0:
            assert rel_l2(leaves_f[k].grad, leaves_d[k].grad) < 1e-4, k


def test_fused_near_plane_culls():
    """A near plane beyond every primitive renders the background only."""
    p = make_params(2000, 6, seed=7)
    cam = S.orbit_view(2, 3.0, 64, 48, 60.0, 60.0, device=DEV)
    bg = torch.tensor([0.3, 0.3, 0.3], device=DEV)
    r = Renderer(dim=6, near_plane=100.0)
    with torch.no_grad():
        colors, alphas = r.render(p, Views([cam], device=DEV), bg)
    assert torch.equal(colors, bg.expand_as(colors)) and not alphas.any()
