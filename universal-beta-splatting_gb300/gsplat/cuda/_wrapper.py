"""Drop-in replacement of the reference's gsplat.cuda._wrapper for the Universal
Beta Splatting rasteriser path, running the GB300 kernels of libubs_gb300.so.

Function names, argument meaning, shapes and autograd behaviour follow
submodules/gsplat/cuda/_wrapper.py of the reference.  Every compute call goes
through the C ABI (include/ubs.h); there is no CPU or PyTorch fallback.

Operators the reference defines but the UBS path never calls
(quat_scale_to_covar_preci, proj, world_to_cam, rasterize_to_indices_in_range)
raise NotImplementedError.
"""
import ctypes
import os
from typing import Optional, Tuple

import torch
from torch import Tensor

from ubs import _lib as L

# Conditioning backward: "reference" reproduces the reference CUDA backward
# (cond_mean_convariance_opacity_bwd.cu), including its transposed Cholesky
# factor; "exact" returns the true gradient of the forward.  The mode in effect
# when the forward runs is the one its backward uses.
_COND_GRAD_MODE = os.environ.get("UBS_COND_GRAD", "reference")

# channel counts with a dedicated kernel; others are padded (as the reference
# does, _wrapper.py:419-464) or split into 32-channel chunks above 33
_NATIVE_CHANNELS = (1, 2, 3, 4, 5, 8, 9, 16, 17, 32, 33)


def set_cond_grad_mode(mode: str) -> None:
    global _COND_GRAD_MODE
    if mode not in ("reference", "exact"):
        raise ValueError("cond grad mode must be 'reference' or 'exact'")
    _COND_GRAD_MODE = mode


def get_cond_grad_mode() -> str:
    return _COND_GRAD_MODE


def _f32(t: Tensor) -> Tensor:
    if t.dtype != torch.float32:
        raise TypeError("the GB300 rasteriser computes in float32; got %s" % t.dtype)
    return t.contiguous()


# --------------------------------------------------------------------- a4
def cond_mean_convariance_opacity(
    means: Tensor,  # [N, D]
    covars: Tensor,  # [N, D, D]
    opacities: Tensor,  # [N, 1]
    betas: Tensor,  # [N, D-3]
    query: Tensor,  # [N, D-3]
) -> Tuple[Tensor, Tensor, Tensor]:
    """Condition mean, covariance and opacity on a query (_wrapper.py:18-31)."""
    return _CondMeanConvarianceOpacity.apply(means.contiguous(), covars.contiguous(),
                                             opacities.contiguous(), betas.contiguous(),
                                             query.contiguous())


class _CondMeanConvarianceOpacity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, covars, opacities, betas, query):
        means, covars, opacities = _f32(means), _f32(covars), _f32(opacities)
        betas, query = _f32(betas), _f32(query)
        N, D = means.shape
        assert covars.shape == (N, D, D), covars.shape
        assert opacities.numel() == N and betas.shape == (N, D - 3) and query.shape == (N, D - 3)
        om = torch.empty(N, 3, device=means.device, dtype=torch.float32)
        oV = torch.empty(N, 3, 3, device=means.device, dtype=torch.float32)
        oo = torch.empty(N, 1, device=means.device, dtype=torch.float32)
        L.call("ubs_cond_fwd", N, D, L.ptr(means), L.ptr(covars), L.ptr(opacities), L.ptr(betas),
               L.ptr(query), L.ptr(om), L.ptr(oV), L.ptr(oo), L.stream(means.device))
        ctx.save_for_backward(means, covars, opacities, betas, query)
        ctx.exact = _COND_GRAD_MODE == "exact"  # the mode at forward time applies
        return om, oV, oo

    @staticmethod
    def backward(ctx, v_m, v_V, v_o):
        means, covars, opacities, betas, query = ctx.saved_tensors
        N, D = means.shape
        dev = means.device
        v_m = torch.zeros(N, 3, device=dev) if v_m is None else _f32(v_m)
        v_V = torch.zeros(N, 3, 3, device=dev) if v_V is None else _f32(v_V)
        v_o = torch.zeros(N, 1, device=dev) if v_o is None else _f32(v_o)
        gm = torch.empty(N, D, device=dev)
        gV = torch.empty(N, D, D, device=dev)
        go = torch.empty(N, 1, device=dev)
        gb = torch.empty(N, D - 3, device=dev)
        L.call("ubs_cond_bwd", N, D, L.ptr(means), L.ptr(covars), L.ptr(opacities), L.ptr(betas),
               L.ptr(query), L.ptr(v_m), L.ptr(v_V), L.ptr(v_o), L.ptr(gm), L.ptr(gV), L.ptr(go),
               L.ptr(gb), 1 if ctx.exact else 0, L.stream(dev))
        return gm, gV, go.view_as(opacities), gb, None


# --------------------------------------------------------------------- a2
def l_triangle_to_rotmat(l_triangle: Tensor) -> Tensor:
    """R = I + A from the 3 skew entries (_wrapper.py:34-36)."""
    assert l_triangle.shape[1] == 3, l_triangle.shape
    return _LTriangleToRotmat.apply(l_triangle.contiguous())


class _LTriangleToRotmat(torch.autograd.Function):
    @staticmethod
    def forward(ctx, l_triangle):
        l_triangle = _f32(l_triangle)
        n = l_triangle.shape[0]
        R = torch.empty(n, 3, 3, device=l_triangle.device)
        L.call("ubs_l_triangle_to_rotmat_fwd", n, L.ptr(l_triangle), l_triangle.shape[1],
               L.ptr(R), L.stream(l_triangle.device))
        ctx.save_for_backward(l_triangle)
        return R

    @staticmethod
    def backward(ctx, v_R):
        (l_triangle,) = ctx.saved_tensors
        v_R = _f32(v_R)
        n = l_triangle.shape[0]
        v_l = torch.empty(n, 3, device=l_triangle.device)
        L.call("ubs_l_triangle_to_rotmat_bwd", n, L.ptr(v_R), L.ptr(v_l),
               L.stream(l_triangle.device))
        return v_l


# --------------------------------------------------------------------- a3
def rot_scale_l_triangle_to_covar(
    rot: Tensor,  # [N, 3, 3]
    scale: Tensor,  # [N, D]
    l_triangle: Tensor,  # [N, D*(D-1)//2]
    rest_i: Tensor,
    rest_j: Tensor,
    spatial_block: bool = False,
) -> Tensor:
    """Sigma = L L^T (_wrapper.py:39-55)."""
    return _RotScaleLTriangleToCovar.apply(rot.contiguous(), scale.contiguous(),
                                           l_triangle.contiguous(), rest_i, rest_j,
                                           spatial_block)


class _RotScaleLTriangleToCovar(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rot, scale, l_triangle, rest_i, rest_j, spatial_block):
        rot, scale, l_triangle = _f32(rot), _f32(scale), _f32(l_triangle)
        N, D = scale.shape
        ri = rest_i.to(device=rot.device, dtype=torch.int32).contiguous()
        rj = rest_j.to(device=rot.device, dtype=torch.int32).contiguous()
        dim = 3 if (spatial_block or D == 3) else D
        covar = torch.empty(N, dim, dim, device=rot.device)
        L.call("ubs_rot_scale_l_triangle_to_covar_fwd", N, D, L.ptr(rot), L.ptr(scale),
               L.ptr(l_triangle), L.ptr(ri), L.ptr(rj), ri.numel(), int(bool(spatial_block)),
               L.ptr(covar), L.stream(rot.device))
        ctx.save_for_backward(rot, scale, l_triangle, ri, rj)
        ctx.spatial_block = bool(spatial_block)
        return covar

    @staticmethod
    def backward(ctx, v_covar):
        rot, scale, l_triangle, ri, rj = ctx.saved_tensors
        if not any(ctx.needs_input_grad[:3]):
            return None, None, None, None, None, None
        N, D = scale.shape
        v_covar = _f32(v_covar)
        v_rot = torch.empty(N, 3, 3, device=rot.device)
        v_scale = torch.empty(N, D, device=rot.device)
        v_l = torch.empty(N, D * (D - 1) // 2, device=rot.device)
        L.call("ubs_rot_scale_l_triangle_to_covar_bwd", N, D, L.ptr(rot), L.ptr(scale),
               L.ptr(l_triangle), L.ptr(ri), L.ptr(rj), ri.numel(), int(ctx.spatial_block),
               L.ptr(v_covar), L.ptr(v_rot), L.ptr(v_scale), L.ptr(v_l), L.stream(rot.device))
        return v_rot, v_scale, v_l, None, None, None


# --------------------------------------------------------------------- a6
def fully_fused_projection(
    means: Tensor,  # [N, 3]
    covars: Optional[Tensor],  # [N, 6] or None
    quats: Optional[Tensor],  # [N, 4] or None
    scales: Optional[Tensor],  # [N, 3] or None
    viewmats: Tensor,  # [C, 4, 4]
    Ks: Tensor,  # [C, 3, 3]
    width: int,
    height: int,
    eps2d: float = 0.3,
    near_plane: float = 0.01,
    far_plane: float = 1e10,
    radius_clip: float = 0.0,
    sparse_grad: bool = False,
    calc_compensations: bool = False,
    ortho: bool = False,
) -> Tuple[Tensor, Tensor, Tensor, Tensor, Tensor]:
    """Projects primitives to 2D (_wrapper.py:185-282).

    Returns radii [C,N] int32, means2d [C,N,2], depths [C,N], conics [C,N,3],
    compensations [C,N] or None.  Culled entries have radius 0 and zeros.
    """
    C = viewmats.size(0)
    N = means.size(0)
    assert means.size() == (N, 3), means.size()
    assert viewmats.size() == (C, 4, 4), viewmats.size()
    assert Ks.size() == (C, 3, 3), Ks.size()
    if ortho:
        raise NotImplementedError("orthographic projection is not on the UBS path")
    if covars is not None:
        assert covars.size() in ((N, 6), (N, 3, 3)), covars.size()
    else:
        assert quats is not None and scales is not None, "covars or quats+scales is required"
        assert quats.size() == (N, 4) and scales.size() == (N, 3)
    return _FullyFusedProjection.apply(
        means.contiguous(), None if covars is None else covars.contiguous(),
        None if quats is None else quats.contiguous(),
        None if scales is None else scales.contiguous(), viewmats.contiguous(), Ks.contiguous(),
        width, height, eps2d, near_plane, far_plane, radius_clip, calc_compensations)


class _FullyFusedProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, covars, quats, scales, viewmats, Ks, width, height, eps2d,
                near_plane, far_plane, radius_clip, calc_compensations):
        means, viewmats, Ks = _f32(means), _f32(viewmats), _f32(Ks)
        layout = 0
        if covars is not None:
            covars = _f32(covars)
            layout = 9 if covars.dim() == 3 else 6
        else:
            quats, scales = _f32(quats), _f32(scales)
        C, N = viewmats.shape[0], means.shape[0]
        dev = means.device
        radii = torch.empty(C, N, dtype=torch.int32, device=dev)
        means2d = torch.empty(C, N, 2, device=dev)
        depths = torch.empty(C, N, device=dev)
        conics = torch.empty(C, N, 3, device=dev)
        comps = torch.empty(C, N, device=dev) if calc_compensations else None
        L.call("ubs_projection_fwd", C, N, L.ptr(means), L.ptr(covars), layout, L.ptr(quats),
               L.ptr(scales), L.ptr(viewmats), L.ptr(Ks), int(width), int(height), float(eps2d),
               float(near_plane), float(far_plane), float(radius_clip), L.ptr(radii),
               L.ptr(means2d), L.ptr(depths), L.ptr(conics), L.ptr(comps), L.stream(dev))
        ctx.save_for_backward(means, covars, quats, scales, viewmats, Ks, radii, conics, comps)
        ctx.layout = layout
        ctx.width, ctx.height, ctx.eps2d = int(width), int(height), float(eps2d)
        ctx.mark_non_differentiable(radii)
        return radii, means2d, depths, conics, comps

    @staticmethod
    def backward(ctx, v_radii, v_means2d, v_depths, v_conics, v_comps):
        means, covars, quats, scales, viewmats, Ks, radii, conics, comps = ctx.saved_tensors
        C, N = viewmats.shape[0], means.shape[0]
        dev = means.device
        zeros = lambda *s: torch.zeros(*s, device=dev)  # noqa: E731
        v_means2d = zeros(C, N, 2) if v_means2d is None else _f32(v_means2d)
        v_depths = zeros(C, N) if v_depths is None else _f32(v_depths)
        v_conics = zeros(C, N, 3) if v_conics is None else _f32(v_conics)
        v_comps = None if (v_comps is None or comps is None) else _f32(v_comps)
        v_means = torch.empty(N, 3, device=dev)
        v_covars = torch.empty_like(covars) if covars is not None else None
        v_quats = torch.empty(N, 4, device=dev) if covars is None else None
        v_scales = torch.empty(N, 3, device=dev) if covars is None else None
        v_view = torch.empty(C, 4, 4, device=dev) if ctx.needs_input_grad[4] else None
        L.call("ubs_projection_bwd", C, N, L.ptr(means), L.ptr(covars), ctx.layout, L.ptr(quats),
               L.ptr(scales), L.ptr(viewmats), L.ptr(Ks), ctx.width, ctx.height, ctx.eps2d,
               L.ptr(radii), L.ptr(conics), L.ptr(comps), L.ptr(v_means2d), L.ptr(v_depths),
               L.ptr(v_conics), L.ptr(v_comps), L.ptr(v_means), L.ptr(v_covars), L.ptr(v_quats),
               L.ptr(v_scales), L.ptr(v_view), L.stream(dev))
        g = ctx.needs_input_grad
        return (v_means if g[0] else None, v_covars if g[1] else None,
                v_quats if g[2] else None, v_scales if g[3] else None,
                v_view if g[4] else None) + (None,) * 8


# --------------------------------------------------------------- a7 / a8
def _isect(means2d, radii, depths, tile_size, tile_width, tile_height, sort=True):
    """Intersections plus the (camera, tile) offsets the count step yields."""
    C, N, _ = means2d.shape
    means2d, depths = _f32(means2d), _f32(depths)
    radii = radii.to(torch.int32).contiguous()
    dev = means2d.device
    st = L.stream(dev)
    n_tiles = int(tile_width) * int(tile_height)
    tpg = torch.empty(C, N, dtype=torch.int32, device=dev)
    offsets = torch.empty(C, int(tile_height), int(tile_width), dtype=torch.int32, device=dev)
    ws = L.workspace(L.query("ubs_isect_count_workspace_bytes", C, N, n_tiles), dev)
    n = ctypes.c_int64(0)
    L.call("ubs_isect_count", C, N, L.ptr(means2d), L.ptr(radii), L.ptr(depths), int(tile_size),
           int(tile_width), int(tile_height), L.ptr(tpg), L.ptr(offsets), ctypes.byref(n),
           L.ptr(ws), ws.numel(), st)
    T = int(n.value)
    isect_ids = torch.empty(T, dtype=torch.int64, device=dev)
    flatten_ids = torch.empty(T, dtype=torch.int32, device=dev)
    if T > 0:
        ws2 = L.workspace(L.query("ubs_isect_sort_workspace_bytes", C, N, n_tiles, T), dev)
        L.call("ubs_isect_emit", C, N, L.ptr(means2d), L.ptr(radii), L.ptr(depths),
               int(tile_size), int(tile_width), int(tile_height), L.ptr(tpg), L.ptr(offsets), T,
               int(bool(sort)), L.ptr(isect_ids), L.ptr(flatten_ids), L.ptr(ws2), ws2.numel(), st)
    return tpg, isect_ids, flatten_ids, offsets


@torch.no_grad()
def isect_tiles(
    means2d: Tensor,  # [C, N, 2]
    radii: Tensor,  # [C, N]
    depths: Tensor,  # [C, N]
    tile_size: int,
    tile_width: int,
    tile_height: int,
    sort: bool = True,
    n_cameras: Optional[int] = None,
    camera_ids: Optional[Tensor] = None,
    primitive_ids: Optional[Tensor] = None,
) -> Tuple[Tensor, Tensor, Tensor]:
    """Maps projected primitives to intersecting tiles (_wrapper.py:286-343).

    Returns tiles_per_gauss [C,N] int32, isect_ids [n_isects] int64
    (camera | tile | depth bits) and flatten_ids [n_isects] int32.
    """
    if camera_ids is not None or primitive_ids is not None:
        raise NotImplementedError("packed intersection input is not on the UBS path")
    C, N, _ = means2d.shape
    assert means2d.shape == (C, N, 2), means2d.size()
    assert radii.shape == (C, N), radii.size()
    assert depths.shape == (C, N), depths.size()
    tpg, ids, fl, _ = _isect(means2d, radii, depths, tile_size, tile_width, tile_height, sort)
    return tpg, ids, fl


@torch.no_grad()
def isect_offset_encode(isect_ids: Tensor, n_cameras: int, tile_width: int,
                        tile_height: int) -> Tensor:
    """First sorted intersection of every (camera, tile) (_wrapper.py:347-363)."""
    isect_ids = isect_ids.to(torch.int64).contiguous()
    dev = isect_ids.device
    offsets = torch.empty(n_cameras, tile_height, tile_width, dtype=torch.int32, device=dev)
    L.call("ubs_isect_offset_encode", isect_ids.numel(), L.ptr(isect_ids), int(n_cameras),
           int(tile_width), int(tile_height), L.ptr(offsets), L.stream(dev))
    return offsets


# ------------------------------------------------------------ a9 / a10
def rasterize_to_pixels(
    means2d: Tensor,  # [C, N, 2]
    conics: Tensor,  # [C, N, 3]
    colors: Tensor,  # [C, N, channels]
    opacities: Tensor,  # [C, N]
    betas: Tensor,  # [C, N]
    image_width: int,
    image_height: int,
    tile_size: int,
    isect_offsets: Tensor,  # [C, tile_height, tile_width]
    flatten_ids: Tensor,  # [n_isects]
    backgrounds: Optional[Tensor] = None,  # [C, channels]
    masks: Optional[Tensor] = None,  # [C, tile_height, tile_width]
) -> Tuple[Tensor, Tensor]:
    """Front-to-back Beta-kernel blend (_wrapper.py:366-491).

    Returns render_colors [C,H,W,channels] and render_alphas [C,H,W,1].
    """
    C = isect_offsets.size(0)
    device = means2d.device
    N = means2d.size(1)
    assert means2d.shape == (C, N, 2), means2d.shape
    assert conics.shape == (C, N, 3), conics.shape
    assert colors.shape[:2] == (C, N), colors.shape
    assert opacities.shape == (C, N), opacities.shape
    assert betas.shape == (C, N), betas.shape
    if backgrounds is not None:
        assert backgrounds.shape == (C, colors.shape[-1]), backgrounds.shape
        backgrounds = backgrounds.contiguous()
    if masks is not None:
        assert masks.shape == isect_offsets.shape, masks.shape
        masks = masks.contiguous()
    channels = colors.shape[-1]
    if channels > 513 or channels == 0:
        raise ValueError(f"Unsupported number of color channels: {channels}")
    tile_height, tile_width = isect_offsets.shape[1:3]
    assert tile_height * tile_size >= image_height, \
        f"Assert Failed: {tile_height} * {tile_size} >= {image_height}"
    assert tile_width * tile_size >= image_width, \
        f"Assert Failed: {tile_width} * {tile_size} >= {image_width}"

    if channels > 33:
        # 32-channel chunks; alphas are identical across chunks and only the
        # first chunk's alphas are returned, so the gradient is unchanged
        outs, alphas = [], None
        for s in range(0, channels, 32):
            cc = colors[..., s:s + 32]
            bb = backgrounds[..., s:s + 32] if backgrounds is not None else None
            o, a = rasterize_to_pixels(means2d, conics, cc, opacities, betas, image_width,
                                       image_height, tile_size, isect_offsets, flatten_ids, bb,
                                       masks)
            outs.append(o)
            alphas = a if alphas is None else alphas
        return torch.cat(outs, dim=-1), alphas

    padded = 0
    if channels not in _NATIVE_CHANNELS:
        padded = (1 << (channels - 1).bit_length()) - channels
        colors = torch.cat([colors, torch.zeros(*colors.shape[:-1], padded, device=device)], -1)
        if backgrounds is not None:
            backgrounds = torch.cat(
                [backgrounds, torch.zeros(*backgrounds.shape[:-1], padded, device=device)], -1)
    render_colors, render_alphas = _RasterizeToPixels.apply(
        means2d.contiguous(), conics.contiguous(), colors.contiguous(), opacities.contiguous(),
        betas.contiguous(), backgrounds, masks, int(image_width), int(image_height),
        int(tile_size), isect_offsets.contiguous(), flatten_ids.contiguous())
    if padded > 0:
        render_colors = render_colors[..., :-padded]
    return render_colors, render_alphas


class _RasterizeToPixels(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means2d, conics, colors, opacities, betas, backgrounds, masks, width,
                height, tile_size, isect_offsets, flatten_ids):
        means2d, conics, colors = _f32(means2d), _f32(conics), _f32(colors)
        opacities, betas = _f32(opacities), _f32(betas)
        if backgrounds is not None:
            backgrounds = _f32(backgrounds)
        mask_u8 = None if masks is None else masks.to(torch.uint8).contiguous()
        offsets = isect_offsets.to(torch.int32).contiguous()
        flatten_ids = flatten_ids.to(torch.int32).contiguous()
        C, N, ch = colors.shape
        T = flatten_ids.numel()
        th, tw = offsets.shape[1:3]
        dev = means2d.device
        render_colors = torch.empty(C, height, width, ch, device=dev)
        render_alphas = torch.empty(C, height, width, 1, device=dev)
        last_ids = torch.empty(C, height, width, dtype=torch.int32, device=dev)
        ws = L.workspace(L.query("ubs_raster_workspace_bytes", T, ch), dev)
        st = L.stream(dev)
        # one record per sorted intersection; the backward reuses the same records
        L.call("ubs_raster_pack", C, N, ch, T, L.ptr(flatten_ids), L.ptr(means2d), L.ptr(conics),
               L.ptr(opacities), L.ptr(betas), L.ptr(colors), L.ptr(ws), ws.numel(), st)
        L.call("ubs_raster_fwd_packed", C, N, ch, T, L.ptr(colors), L.ptr(backgrounds),
               L.ptr(mask_u8), width, height, tile_size, tw, th, L.ptr(offsets),
               L.ptr(render_colors), L.ptr(render_alphas), L.ptr(last_ids), 0, L.ptr(ws),
               ws.numel(), st)
        ctx.ws = ws
        ctx.save_for_backward(means2d, conics, colors, opacities, betas, backgrounds, mask_u8,
                              offsets, flatten_ids, render_alphas, last_ids)
        ctx.width, ctx.height, ctx.tile_size = width, height, tile_size
        ctx.mark_non_differentiable(last_ids)
        return render_colors, render_alphas

    @staticmethod
    def backward(ctx, v_render_colors, v_render_alphas):
        (means2d, conics, colors, opacities, betas, backgrounds, mask_u8, offsets, flatten_ids,
         render_alphas, last_ids) = ctx.saved_tensors
        C, N, ch = colors.shape
        T = flatten_ids.numel()
        th, tw = offsets.shape[1:3]
        dev = means2d.device
        if v_render_colors is None:
            v_render_colors = torch.zeros(C, ctx.height, ctx.width, ch, device=dev)
        if v_render_alphas is None:
            v_render_alphas = torch.zeros(C, ctx.height, ctx.width, 1, device=dev)
        v_render_colors = _f32(v_render_colors)
        v_render_alphas = _f32(v_render_alphas)
        v_means2d = torch.zeros_like(means2d)
        v_conics = torch.zeros_like(conics)
        v_colors = torch.zeros_like(colors)
        v_opacities = torch.zeros_like(opacities)
        v_betas = torch.zeros_like(betas)
        ws = ctx.ws
        L.call("ubs_raster_bwd_packed", C, N, ch, T, L.ptr(colors), L.ptr(backgrounds),
               L.ptr(mask_u8), ctx.width, ctx.height, ctx.tile_size, tw, th, L.ptr(offsets),
               L.ptr(render_alphas), L.ptr(last_ids), L.ptr(v_render_colors),
               L.ptr(v_render_alphas), L.ptr(v_means2d), L.ptr(v_conics), L.ptr(v_colors),
               L.ptr(v_opacities), L.ptr(v_betas), 0, L.ptr(ws), ws.numel(), L.stream(dev))
        ctx.ws = None
        v_backgrounds = None
        if ctx.needs_input_grad[5]:
            v_backgrounds = (v_render_colors * (1.0 - render_alphas).float()).sum(dim=(1, 2))
        return (v_means2d, v_conics, v_colors, v_opacities, v_betas, v_backgrounds) + (None,) * 6


# ------------------------------------------- operators outside the UBS path
def _not_on_path(name):
    def f(*args, **kwargs):
        raise NotImplementedError(
            "%s is part of the reference's generic gsplat operator set but is never called on "
            "the Universal Beta Splatting rasteriser path" % name)
    f.__name__ = name
    return f


quat_scale_to_covar_preci = _not_on_path("quat_scale_to_covar_preci")
persp_proj = _not_on_path("persp_proj")
proj = _not_on_path("proj")
world_to_cam = _not_on_path("world_to_cam")
rasterize_to_indices_in_range = _not_on_path("rasterize_to_indices_in_range")
