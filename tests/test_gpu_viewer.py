"""The viewer frame (ubs.viewer) against the reference's BetaModel.view steps
(scene/beta_model.py:725-831) restated with torch.quantile, masked gathers
and the drop-in rasterization(): Beta quantile masks and bounds exact,
colormap lookups exact, frames within the rasteriser's 1e-5 (depth 3e-5)."""
import math
import types

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from gsplat.cuda._wrapper import (cond_mean_convariance_opacity, l_triangle_to_rotmat,
                                  rot_scale_l_triangle_to_covar)
from gsplat.rendering import rasterization
from ubs import scene as S
from ubs.viewer import FrameRenderer, ViewState, view

pytestmark = pytest.mark.gpu
DEV = "cuda"
W, H = 320, 240


def ref_quantile_mask(beta, b_xyz, b_view, b_time):
    """quantile_mask of BetaModel.view, in torch."""
    x = beta[:, 0]
    v = beta[:, 1:4].mean(dim=-1)
    m = ((x >= x.quantile(b_xyz[0] / 100)) & (x <= x.quantile(b_xyz[1] / 100))
         & (v >= v.quantile(b_view[0] / 100)) & (v <= v.quantile(b_view[1] / 100)))
    if b_time is not None:
        t = beta[:, 4]
        m = m & (t >= t.quantile(b_time[0] / 100)) & (t <= t.quantile(b_time[1] / 100))
    return m


def ref_colormap(img, table):
    """apply_depth_colormap + apply_float_colormap with a given table."""
    near, far = float(torch.min(img)), float(torch.max(img))
    d = torch.clip((img - near) / (far - near + 1e-10), 0.0, 1.0)
    d = torch.nan_to_num(d, 0)
    return table[(d * 255).long()[..., 0]]


def camera(seed=0):
    cam = S.orbit_view(seed, 3.0, W, H, 300.0, 300.0)
    c2w = torch.inverse(cam.viewmat.cpu()).numpy()
    K = cam.K.cpu().numpy()
    return c2w, K


def ref_frame(p, c2w, K, state, dim):
    """BetaModel.view's render for one frame: mask, condition, rasterize."""
    c2w_t = torch.from_numpy(c2w).float().to(DEV)
    K_t = torch.from_numpy(K).float().to(DEV)
    mask = ref_quantile_mask(p["beta"], state.b_xyz, state.b_view,
                             state.b_time if dim == 7 else None)
    cam_pos = c2w_t[:3, 3]
    view_dir = p["xyz"] - cam_pos[None]
    query = view_dir / view_dir.norm(dim=-1, keepdim=True)
    if dim == 7:
        query = torch.cat([query, torch.full_like(query[:, :1], state.timestamp)], -1)
    scale = F.softplus(p["scale"])
    beta = 4.0 * torch.exp(p["beta"])
    ri, rj = S.rest_indices(dim, DEV)
    R = l_triangle_to_rotmat(p["l_triangle"][:, :3])
    cov = rot_scale_l_triangle_to_covar(R, scale, p["l_triangle"], ri, rj)
    means, convs, opac = cond_mean_convariance_opacity(
        torch.cat([p["xyz"], p["mean"]], -1), cov, torch.sigmoid(p["opacity"]), beta[:, 1:],
        query)
    bg = torch.tensor(state.backgrounds, device=DEV) / 255.0
    mode = state.render_mode
    rc, ra, meta = rasterization(
        means=means[mask], l_triagnles=p["l_triangle"][mask], scales=scale[mask],
        opacities=opac.squeeze()[mask], betas=beta[:, :1].squeeze()[mask], colors=p["rgb"][mask],
        viewmats=torch.linalg.inv(c2w_t)[None], Ks=K_t[None], width=W, height=H,
        backgrounds=bg[None], render_mode=mode if mode != "Alpha" else "RGB", covars=convs[mask],
        near_plane=state.near_plane, far_plane=state.far_plane, radius_clip=state.radius_clip)
    if mode == "Alpha":
        rc = ra
    return rc[0], mask, int((meta["radii"] > 0).sum())


def scene(N, dim, seed=0):
    p = S.synthetic_params(N, dim, seed=seed, xyz_range=1.0, device=DEV)
    with torch.no_grad():  # bigger, more visible primitives for a 320x240 frame
        p["scale"][:, :3] += 1.5
    return p


@pytest.mark.parametrize("dim", [6, 7])
@pytest.mark.parametrize("ranges", [((0, 100), (0, 100), (0, 100)), ((5, 95), (10, 90), (0, 60)),
                                    ((37, 38), (0, 100), (50, 100)), ((0, 0), (100, 100), (0, 1))])
def test_quantile_mask_and_bounds_exact(dim, ranges):
    g = torch.Generator().manual_seed(dim)
    N = 100_003
    beta = torch.randn(N, dim - 2, generator=g)
    beta[: N // 3] = torch.round(beta[: N // 3] * 8) / 8  # many ties
    beta = beta.to(DEV)
    fr = FrameRenderer(dim=dim, table=torch.zeros(256, 3))
    st = ViewState(b_xyz=ranges[0], b_view=ranges[1], b_time=ranges[2])
    got = fr.quantile_mask(beta, st).bool()
    want = ref_quantile_mask(beta, st.b_xyz, st.b_view, st.b_time if dim == 7 else None)
    assert torch.equal(got, want), (got.sum().item(), want.sum().item())
    import ctypes
    from ubs import _lib as L
    n_arr = 3 if dim == 7 else 2
    bounds = torch.empty(2 * n_arr, device=DEV)
    L.call("ubs_quantile_mask_bounds", L.ptr(fr._qws), n_arr, L.ptr(bounds), L.stream(DEV))
    arrays = [beta[:, 0], beta[:, 1:4].mean(dim=-1)] + ([beta[:, 4]] if dim == 7 else [])
    want_b = []
    for a, (lo, hi) in zip(arrays, ranges):
        want_b += [a.quantile(lo / 100).item(), a.quantile(hi / 100).item()]
    assert bounds.cpu().tolist() == want_b
    del ctypes


def test_quantile_mask_nan_gives_empty_mask():
    beta = torch.randn(1000, 4, device=DEV)
    beta[17, 0] = float("nan")
    fr = FrameRenderer(dim=6, table=torch.zeros(256, 3))
    got = fr.quantile_mask(beta, ViewState())
    assert not got.any()
    assert not ref_quantile_mask(beta, (0, 100), (0, 100), None).any()


def test_colormap_exact():
    g = torch.Generator().manual_seed(3)
    table = torch.rand(256, 3, generator=g).to(DEV)
    fr = FrameRenderer(dim=6, table=table)
    for img in (torch.rand(H, W, 1, generator=g) * 7 + 2, torch.zeros(5, 7, 1),
                torch.linspace(0, 1, 1000).view(10, 100, 1)):
        img = img.to(DEV)
        assert torch.equal(fr.colormap(img), ref_colormap(img, table))


@pytest.mark.parametrize("dim", [6, 7])
@pytest.mark.parametrize("mode", ["RGB", "Alpha", "Depth", "Normal"])
def test_frame_matches_reference_view(dim, mode):
    p = scene(20_000, dim, seed=dim)
    c2w, K = camera(dim)
    g = torch.Generator().manual_seed(5)
    table = torch.rand(256, 3, generator=g).to(DEV)
    fr = FrameRenderer(dim=dim, table=table)
    st = ViewState(b_xyz=(3, 97), b_view=(2, 90), b_time=(0, 80), backgrounds=(30, 60, 90),
                   render_mode=mode, near_plane=0.01, far_plane=100.0, timestamp=0.3)
    img = torch.from_numpy(fr.render(p, c2w, K, W, H, st, copy=True))
    dimg, raw, _ = fr.frame(p, c2w, K, W, H, st)
    assert torch.equal(dimg.cpu(), img)
    ref_st = ViewState(**{**st.__dict__, "render_mode": "Depth" if mode == "Normal" else mode})
    ref, mask, n_vis = ref_frame(p, c2w, K, ref_st, dim)
    assert fr.rendered_count == n_vis and fr.total_count == 20_000
    # the rendered channels (depth: FP32 accumulation of values ~3, 3e-5)
    tol = 3e-5 if mode in ("Depth", "Normal") else 1e-5
    err = (raw - ref).abs() / torch.clamp(ref.abs(), min=1.0)
    assert float(err.max()) < tol
    if mode == "Normal":  # exactly the reference's normals of that depth
        from gsplat.utils import depth_to_normal
        vm = torch.linalg.inv(torch.from_numpy(c2w).float())[None].to(DEV)
        want = (depth_to_normal(raw[None], torch.inverse(vm),
                                torch.from_numpy(K).float()[None].to(DEV)) + 1) / 2
        assert torch.equal(dimg, want[0])
    elif mode in ("Alpha", "Depth"):  # exactly the reference's colormap of that image
        assert torch.equal(dimg, ref_colormap(raw, table))


def test_view_drop_in():
    p = scene(5000, 6, seed=9)
    c2w, K = camera(9)
    model = types.SimpleNamespace(input_dim=6, **{"_" + k: torch.nn.Parameter(v)
                                                   for k, v in p.items()})
    cam = types.SimpleNamespace(c2w=c2w, get_K=lambda wh: K)
    tab = types.SimpleNamespace(preview_render=False, viewer_width=W, viewer_height=H,
                                timestamp=0.0, near_plane=1e-3, far_plane=1e3, radius_clip=0.0,
                                b_xyz=(0, 100), b_view=(0, 100), b_time=(0, 100),
                                backgrounds=(0, 0, 0), render_mode="RGB")
    img = view(model, cam, tab)
    assert img.shape == (H, W, 3) and img.dtype == np.float32
    assert tab.total_count_number == 5000 and 0 < tab.rendered_count_number <= 5000
    img2 = view(model, cam, tab)
    assert np.array_equal(img, img2)


def test_empty_scene_frame():
    p = {k: v[:0] for k, v in scene(10, 6).items()}
    c2w, K = camera(1)
    fr = FrameRenderer(dim=6, table=torch.zeros(256, 3))
    img = fr.render(p, c2w, K, W, H, ViewState(backgrounds=(51, 102, 153)), copy=True)
    want = np.array([51, 102, 153], np.float32) / np.float32(255.0)
    assert np.array_equal(img, np.broadcast_to(want, img.shape))
    assert fr.rendered_count == 0 and fr.total_count == 0
