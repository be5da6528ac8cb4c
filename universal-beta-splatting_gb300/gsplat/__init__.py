"""GB300-native drop-in for the reference's `gsplat` package on the Universal
Beta Splatting rasteriser path (same import names as the reference)."""
from .cuda._wrapper import (
    cond_mean_convariance_opacity,
    fully_fused_projection,
    isect_offset_encode,
    isect_tiles,
    l_triangle_to_rotmat,
    proj,
    quat_scale_to_covar_preci,
    rasterize_to_indices_in_range,
    rasterize_to_pixels,
    rot_scale_l_triangle_to_covar,
    world_to_cam,
)
from .rendering import rasterization

__version__ = "0.1.0+gb300"

__all__ = [
    "rasterization",
    "isect_offset_encode",
    "isect_tiles",
    "proj",
    "fully_fused_projection",
    "quat_scale_to_covar_preci",
    "rasterize_to_pixels",
    "world_to_cam",
    "rasterize_to_indices_in_range",
    "l_triangle_to_rotmat",
    "rot_scale_l_triangle_to_covar",
    "cond_mean_convariance_opacity",
]
