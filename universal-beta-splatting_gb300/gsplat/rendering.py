"""rasterization(): the reference's pipeline entry point
(submodules/gsplat/rendering.py:17-232) on the GB300 kernels.

Same signature, outputs and `meta` keys.  Differences that do not change
results: the covariance upper-triangle gather is fused into the projection
kernel (same gradient), and the (camera, tile) offsets come out of the
intersection count instead of a separate encode pass (same values).
"""
import math
from typing import Dict, Optional, Tuple

import torch
from torch import Tensor
from typing_extensions import Literal

from .cuda._wrapper import _isect, fully_fused_projection, rasterize_to_pixels
from .utils import depth_to_normal

RENDER_MODES = ("RGB", "Normal", "Diffuse", "Specular", "Depth", "EDepth", "RGB+D", "RGB+ED")


def rasterization(
    means: Tensor,  # [N, 3]
    l_triagnles: Tensor,  # [N, 4] (quaternions, used only when covars is None)
    scales: Tensor,  # [N, 3]
    opacities: Tensor,  # [N]
    betas: Tensor,  # [N]
    colors: Tensor,  # [(C,) N, D]
    viewmats: Tensor,  # [C, 4, 4]
    Ks: Tensor,  # [C, 3, 3]
    width: int,
    height: int,
    near_plane: float = 0.01,
    far_plane: float = 1e10,
    radius_clip: float = 0.0,
    eps2d: float = 0.3,
    tile_size: int = 16,
    backgrounds: Optional[Tensor] = None,
    render_mode: Literal[
        "RGB", "Normal", "Diffuse", "Specular", "Depth", "EDepth", "RGB+D", "RGB+ED"
    ] = "RGB",
    rasterize_mode: Literal["classic", "antialiased"] = "classic",
    channel_chunk: int = 32,
    covars: Optional[Tensor] = None,
) -> Tuple[Tensor, Tensor, Dict]:
    meta = {}
    N = means.shape[0]
    C = viewmats.shape[0]
    assert means.shape == (N, 3), means.shape
    if covars is None:
        assert l_triagnles.shape == (N, 4), l_triagnles.shape
        assert scales.shape == (N, 3), scales.shape
    else:
        assert covars.shape == (N, 3, 3), covars.shape
        l_triagnles, scales = None, None
    assert opacities.shape == (N,), opacities.shape
    assert betas.shape == (N,), betas.shape
    assert viewmats.shape == (C, 4, 4), viewmats.shape
    assert Ks.shape == (C, 3, 3), Ks.shape
    assert render_mode in RENDER_MODES, render_mode
    assert (colors.dim() == 2 and colors.shape[0] == N) or (
        colors.dim() == 3 and colors.shape[:2] == (C, N)
    ), colors.shape

    # the upper-triangle gather of the reference happens inside the kernel
    radii, means2d, depths, conics, compensations = fully_fused_projection(
        means, covars, l_triagnles, scales, viewmats, Ks, width, height, eps2d=eps2d,
        near_plane=near_plane, far_plane=far_plane, radius_clip=radius_clip, sparse_grad=False,
        calc_compensations=(rasterize_mode == "antialiased"), ortho=False)
    opacities = opacities.repeat(C, 1)  # [C, N]
    betas = betas.repeat(C, 1)  # [C, N]
    camera_ids, primitive_ids = None, None
    if compensations is not None:
        opacities = opacities * compensations
    meta.update({
        "camera_ids": camera_ids,
        "primitive_ids": primitive_ids,
        "radii": radii,
        "means2d": means2d,
        "depths": depths,
        "conics": conics,
        "opacities": opacities,
        "betas": betas,
    })

    if colors.dim() == 2:
        colors = colors.expand(C, -1, -1)
    if render_mode in ("RGB+D", "RGB+ED"):
        colors = torch.cat((colors, depths[..., None]), dim=-1)
        if backgrounds is not None:
            backgrounds = torch.cat(
                [backgrounds, torch.zeros(C, 1, device=backgrounds.device)], dim=-1)
    elif render_mode in ("Depth", "EDepth", "Normal"):
        colors = depths[..., None]
        if backgrounds is not None:
            backgrounds = torch.zeros(C, 1, device=backgrounds.device)

    tile_width = math.ceil(width / float(tile_size))
    tile_height = math.ceil(height / float(tile_size))
    tiles_per_gauss, isect_ids, flatten_ids, isect_offsets = _isect(
        means2d.detach(), radii, depths.detach(), tile_size, tile_width, tile_height, sort=True)
    meta.update({
        "tile_width": tile_width,
        "tile_height": tile_height,
        "tiles_per_gauss": tiles_per_gauss,
        "isect_ids": isect_ids,
        "flatten_ids": flatten_ids,
        "isect_offsets": isect_offsets,
        "width": width,
        "height": height,
        "tile_size": tile_size,
        "n_cameras": C,
    })

    if colors.shape[-1] > channel_chunk:
        n_chunks = (colors.shape[-1] + channel_chunk - 1) // channel_chunk
        render_colors, render_alphas = [], []
        for i in range(n_chunks):
            cc = colors[..., i * channel_chunk:(i + 1) * channel_chunk]
            bb = (backgrounds[..., i * channel_chunk:(i + 1) * channel_chunk]
                  if backgrounds is not None else None)
            rc, ra = rasterize_to_pixels(means2d, conics, cc, opacities, betas, width, height,
                                         tile_size, isect_offsets, flatten_ids, backgrounds=bb)
            render_colors.append(rc)
            render_alphas.append(ra)
        render_colors = torch.cat(render_colors, dim=-1)
        render_alphas = render_alphas[0]
    else:
        render_colors, render_alphas = rasterize_to_pixels(
            means2d, conics, colors, opacities, betas, width, height, tile_size, isect_offsets,
            flatten_ids, backgrounds=backgrounds)
    # the reference tests for the mode name "ED", so only "RGB+ED" is normalised
    if render_mode in ("ED", "RGB+ED"):
        render_colors = torch.cat(
            [render_colors[..., :-1], render_colors[..., -1:] / render_alphas.clamp(min=1e-10)],
            dim=-1)
    if render_mode == "Normal":
        camtoworlds = torch.inverse(viewmats)
        render_colors = depth_to_normal(render_colors, camtoworlds, Ks)
        render_colors = (render_colors + 1) / 2
    return render_colors, render_alphas, meta
