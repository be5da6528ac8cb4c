"""rasterization(): the entry point the Universal Beta Splatting model calls
(submodules/gsplat/rendering.py:17-232), on the GB300 kernels.

The call surface is the reference's: the same signature and argument
checks, the same outputs and the same `meta` keys.  The body is organised
around a render-mode table instead of branches: each mode names which
per-primitive features are blended (the colours, the camera-space depth or
both), whether the depth channel is divided by the alpha afterwards and
whether the blended depth is turned into normals.  Everything else is one
pass: projection (the upper-triangle gather of a 3x3 covariance happens
inside the projection kernel), one intersection call that also yields the
tile offsets, one blend.  The 32-channel chunking of wide feature rows
lives in `rasterize_to_pixels` (channels blend independently, so the
`channel_chunk` width does not change any result).
"""
import math
from typing import Dict, NamedTuple, Optional, Tuple

import torch
from torch import Tensor
from typing_extensions import Literal

from .cuda._wrapper import _isect, fully_fused_projection, rasterize_to_pixels
from .utils import depth_to_normal


class _Mode(NamedTuple):
    colors: bool           # blend the caller's colour channels
    depth: bool            # blend the camera-space depth as one more channel
    depth_over_alpha: bool  # divide that channel by the alpha afterwards
    normals: bool          # turn the blended depth into world-space normals


# Per render mode.  The reference divides by the alpha only when the mode
# string contains "ED" *and* is tested against "ED"/"RGB+ED" -- "EDepth" is
# not in that list (rendering.py:219), so "EDepth" returns the plain
# accumulated depth; the table keeps that behaviour.
_MODES: Dict[str, _Mode] = {
    "RGB": _Mode(True, False, False, False),
    "Diffuse": _Mode(True, False, False, False),
    "Specular": _Mode(True, False, False, False),
    "Depth": _Mode(False, True, False, False),
    "EDepth": _Mode(False, True, False, False),
    "Normal": _Mode(False, True, False, True),
    "RGB+D": _Mode(True, True, False, False),
    "RGB+ED": _Mode(True, True, True, False),
}
RENDER_MODES = tuple(_MODES)


def _features(mode: _Mode, colors: Tensor, depths: Tensor, backgrounds: Optional[Tensor],
              C: int) -> Tuple[Tensor, Optional[Tensor]]:
    """Per-(camera, primitive) feature rows [C, N, F] and their backgrounds
    [C, F] (None if the caller gave none) for one render mode.  The depth
    channel's background is 0."""
    rows, bgs = [], []
    if mode.colors:
        rows.append(colors if colors.dim() == 3 else colors.unsqueeze(0).expand(C, -1, -1))
        bgs.append(backgrounds)
    if mode.depth:
        rows.append(depths.unsqueeze(-1))
        if backgrounds is not None:
            bgs.append(backgrounds.new_zeros(C, 1))
    feats = rows[0] if len(rows) == 1 else torch.cat(rows, dim=-1)
    if backgrounds is None:
        return feats, None
    return feats, (bgs[0] if len(bgs) == 1 else torch.cat(bgs, dim=-1))


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
    N, C = means.shape[0], viewmats.shape[0]
    # the reference's argument checks (rendering.py:43-70)
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
    assert render_mode in _MODES, render_mode
    assert (colors.dim() == 2 and colors.shape[0] == N) or (
        colors.dim() == 3 and colors.shape[:2] == (C, N)
    ), colors.shape
    assert channel_chunk > 0, channel_chunk
    mode = _MODES[render_mode]

    radii, means2d, depths, conics, comp = fully_fused_projection(
        means, covars, l_triagnles, scales, viewmats, Ks, width, height, eps2d=eps2d,
        near_plane=near_plane, far_plane=far_plane, radius_clip=radius_clip, sparse_grad=False,
        calc_compensations=rasterize_mode == "antialiased", ortho=False)
    # per-camera opacities (antialiased: scaled by the footprint compensation)
    # and betas, [C, N]
    opac_c = opacities.unsqueeze(0).expand(C, N)
    if comp is not None:
        opac_c = opac_c * comp
    betas_c = betas.unsqueeze(0).expand(C, N)

    tiles_x = math.ceil(width / float(tile_size))
    tiles_y = math.ceil(height / float(tile_size))
    tiles_per_gauss, isect_ids, flatten_ids, isect_offsets = _isect(
        means2d.detach(), radii, depths.detach(), tile_size, tiles_x, tiles_y, sort=True)

    feats, feat_bg = _features(mode, colors, depths, backgrounds, C)
    image, alpha = rasterize_to_pixels(means2d, conics, feats, opac_c, betas_c, width, height,
                                       tile_size, isect_offsets, flatten_ids,
                                       backgrounds=feat_bg)
    if mode.depth_over_alpha:
        image = torch.cat([image[..., :-1], image[..., -1:] / alpha.clamp(min=1e-10)], dim=-1)
    if mode.normals:
        image = (depth_to_normal(image, torch.inverse(viewmats), Ks) + 1) / 2

    meta = {
        "camera_ids": None, "primitive_ids": None,
        "radii": radii, "means2d": means2d, "depths": depths, "conics": conics,
        "opacities": opac_c, "betas": betas_c,
        "tile_width": tiles_x, "tile_height": tiles_y,
        "tiles_per_gauss": tiles_per_gauss, "isect_ids": isect_ids,
        "flatten_ids": flatten_ids, "isect_offsets": isect_offsets,
        "width": width, "height": height, "tile_size": tile_size, "n_cameras": C,
    }
    return image, alpha, meta
